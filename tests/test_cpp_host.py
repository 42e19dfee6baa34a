"""The C++ layer (include/nr_gpu_ldpc_gb300.hpp) from a reference-style host
program: it compiles and links against the in-tree library with plain g++
(CPU), and its decode equals the oracle's (GPU)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from nr_gpu_ldpc_gb300 import codes
from oracle.oracle import OracleCode

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build(tmp_path, cuda_lib, name="host_decode", std="c++17"):
    exe = str(tmp_path / name)
    cmd = ["g++", f"-std={std}", "-O2", os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-o", exe,
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           "-L", os.path.join(ROOT, "nr_gpu_ldpc_gb300"), "-lnrldpc_gb300",
           "-Wl,-rpath," + os.path.join(ROOT, "nr_gpu_ldpc_gb300"),
           "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64")]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not present")
def test_cpp_caller_compiles_and_links(tmp_path, cuda_lib):
    assert os.path.exists(_build(tmp_path, cuda_lib))
    # the reference builds as C++14: the compat layer of the header compiles there
    assert os.path.exists(_build(tmp_path, cuda_lib, "compat_decode", "c++14"))


@pytest.mark.gpu
def test_cpp_caller_decodes_like_the_oracle(tmp_path, cuda_lib):
    exe = _build(tmp_path, cuda_lib)
    oc = OracleCode(codes.base_matrix(1, codes.set_index(384)), 384)
    sig = np.full(6, codes.noise_sigma(1.7, 1 / 3), np.float32)
    llr, _ = oc.gen_llr(22, 5150, 0, sig, 2)
    src, dst = tmp_path / "llr.f32", tmp_path / "out.u8"
    llr.tofile(src)
    want, _, _ = oc.minsum_f32(llr, 10)
    for mode in ([], ["0"], ["1"], ["2"]):  # default, AUTO, COPY, DIRECT host transfer
        dst.unlink(missing_ok=True)
        r = subprocess.run([exe, "8424", "10", str(src), str(dst), *mode], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        got = np.fromfile(dst, np.uint8).reshape(want.shape)
        np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
def test_reference_call_shape_decodes_like_the_oracle(tmp_path, cuda_lib):
    """perform_gpu_ldpc_decoding with the reference's arguments (structs with
    its member names, a grid, the stream index) through nrldpc::compat, two
    streams."""
    exe = _build(tmp_path, cuda_lib, "compat_decode", "c++14")
    oc = OracleCode(codes.base_matrix(1, codes.set_index(384)), 384)
    sig = np.full(5, codes.noise_sigma(1.7, 1 / 3), np.float32)
    llr, _ = oc.gen_llr(22, 5151, 0, sig, 2)
    src, dst = tmp_path / "llr.f32", tmp_path / "out.u8"
    llr.tofile(src)
    r = subprocess.run([exe, str(src), str(dst)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    want, _, _ = oc.minsum_f32(llr, 10)
    np.testing.assert_array_equal(np.fromfile(dst, np.uint8).reshape(want.shape), want)


@pytest.mark.gpu
def test_cpp_caller_two_lane_pipeline(tmp_path, cuda_lib):
    """The C++ caller on a batch of more than one CTA round with staged copies:
    the chunks decode on both of the handle's lanes (the caller's stream and
    the handle's own), and the packed bits equal the device-resident decode
    of the same LLRs."""
    import torch
    from nr_gpu_ldpc_gb300 import Decoder
    exe = _build(tmp_path, cuda_lib)
    n = 330  # BG1 Z=384 on a GB300: a 304-codeword round, then 26 more
    dec = Decoder(bg=1, z=384, max_batch=n)
    sig = torch.full((n,), codes.noise_sigma(1.7, 1 / 3), device="cuda")
    llr, _ = dec.gen_llr(71, 0, sig)
    want = dec.decode(llr, 10).cpu().numpy()
    dec.close()
    src, dst = tmp_path / "llr.f32", tmp_path / "out.u8"
    llr.cpu().numpy().tofile(src)
    r = subprocess.run([exe, "8424", "10", str(src), str(dst), "1"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(np.fromfile(dst, np.uint8).reshape(want.shape), want)
