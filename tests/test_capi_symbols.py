"""The C-ABI library loads and exports every entry point the public header
declares; host-only entry points work without a GPU."""
import ctypes as C
import os
import re

from nr_gpu_ldpc_gb300 import _lib, codes

HEADER_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include")


def declared_symbols():
    names = set()
    for f in os.listdir(HEADER_DIR):
        if f.endswith(".h"):
            text = open(os.path.join(HEADER_DIR, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(nrldpc_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(cuda_lib):
    names = declared_symbols()
    assert "nrldpc_decode" in names and len(names) >= 15
    for n in names:
        assert hasattr(cuda_lib, n), n
    assert set(_lib.SIGNATURES) == names


def test_setup_ldpc_c_matches_python(cuda_lib, golden):
    p = _lib.LdpcParamsC()
    for row in golden["setup_ldpc"]:
        assert cuda_lib.nrldpc_setup_ldpc(row["A"], row["rate"], 5, C.byref(p)) == 0
        py = codes.setup_ldpc(row["A"], row["rate"], 5)
        for k in ("A", "bg_index", "Z", "K", "N", "H_rows", "H_cols", "n_nz_in_row", "n_nz_in_col",
                  "N_before_puncture"):
            assert getattr(p, k) == row[k] == getattr(py, k), (row, k)
        assert p.i_ls == py.i_ls and p.C == py.C and p.K_b == py.K_b


def test_setup_ldpc_rejects_unliftable():
    p = _lib.LdpcParamsC()
    lib = _lib.load()
    # BG2 at rate 0.2 with a two-block payload needs Z > 384: the reference
    # would read an uninitialized set index here
    assert lib.nrldpc_setup_ldpc(8000, 0.2, 5, C.byref(p)) == -2


def test_status_strings(cuda_lib):
    assert cuda_lib.nrldpc_status_string(0) == b"ok"
    assert b"aligned" in cuda_lib.nrldpc_status_string(-4)
