"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
and nowhere else.  ``RefEmu`` loads oracle/_ref (the reference's own kernel
source run on the CPU), which exists only where the reference tree was
present at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_lib = None


REF_GPU_CUBIN = os.path.join(REF_DIR, "ref_kernels_bg1.cubin")
REF_GPU_CONST = os.path.join(REF_DIR, "ref_const_bg1.bin")
REF_GPU_LIB = os.path.join(HERE, "_build", "libref_gpu.so")


def build(reference_root: str | None = None, quiet: bool = True) -> None:
    """Run oracle/Makefile (the oracle and the GPU driver of the reference's
    kernels, plus oracle/_ref if the reference exists), then write the
    constant-memory image of the reference's own setup for BG1 Z=384 next to
    its GPU kernels (oracle/_ref/ref_const_bg1.bin)."""
    cmd = ["make", "-C", HERE]
    if reference_root:
        cmd.append(f"REF={reference_root}")
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL if quiet else None)
    if RefEmu.available("bg1") and os.path.exists(REF_GPU_CUBIN):
        # the table of the reference's own configuration: BG1, lifting set 1, Z = 384
        base = _bg1_ils1_base()
        img = RefEmu(base, 384).constant_image()
        with open(REF_GPU_CONST, "wb") as f:
            f.write(img)


def _bg1_ils1_base() -> np.ndarray:
    import sys
    root = os.path.dirname(HERE)
    if root not in sys.path:
        sys.path.insert(0, root)
    from nr_gpu_ldpc_gb300 import codes
    return codes.base_matrix(1, codes.set_index(384))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            subprocess.run(["make", "-C", HERE, os.path.join("_build", "liboracle.so")],
                           check=True, stdout=subprocess.DEVNULL)
        L = C.CDLL(LIB_PATH)
        L.orc_code_new.restype = C.c_void_p
        L.orc_code_new.argtypes = [_i32p, C.c_int, C.c_int, C.c_int]
        L.orc_code_free.argtypes = [C.c_void_p]
        L.orc_code_edges.argtypes = [C.c_void_p]
        L.orc_set_fma_dt.argtypes = [C.c_int]
        L.orc_minsum_f32.argtypes = [C.c_void_p, _f32p, C.c_int, C.c_int, C.c_float, C.c_int,
                                     _u8p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_minsum_f64.argtypes = [C.c_void_p, _f64p, C.c_int, C.c_int, C.c_double, C.c_int,
                                     _u8p, C.c_void_p, C.c_void_p]
        L.orc_syndrome_weight.argtypes = [C.c_void_p, _u8p]
        L.orc_encode.argtypes = [C.c_void_p, C.c_int, _u8p, _u8p]
        L.orc_gen_llr.argtypes = [C.c_void_p, C.c_int, C.c_uint64, C.c_uint64, C.c_int, _f32p,
                                  C.c_int, _f32p, C.c_void_p]
        L.orc_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                     C.POINTER(C.c_uint32)]
        L.orc_logf.restype = C.c_float
        L.orc_logf.argtypes = [C.c_float]
        L.orc_sincos2pi.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_wms_loss_grad_f64.restype = C.c_double
        L.orc_wms_loss_grad_f64.argtypes = [C.c_void_p, _f32p, _u8p, C.c_int, C.c_int, _f64p,
                                            C.c_void_p, C.c_void_p]
        L.orc_wms_layered_loss_grad_f64.restype = C.c_double
        L.orc_wms_layered_loss_grad_f64.argtypes = [C.c_void_p, _f32p, _u8p, C.c_int, C.c_int, _f64p,
                                                    C.c_void_p, C.c_void_p]
        L.orc_wms_layered_loss_grad.restype = C.c_double
        L.orc_wms_layered_loss_grad.argtypes = [C.c_void_p, _f32p, _u8p, C.c_int, C.c_int, _f64p,
                                                C.c_void_p, C.c_void_p, C.c_int]
        L.orc_wms_decode_f32.argtypes = [C.c_void_p, _f32p, C.c_int, C.c_int, _f32p, C.c_int,
                                         C.c_int, _u8p, C.c_void_p, C.c_void_p]
        L.orc_layered_f32.argtypes = [C.c_void_p, _f32p, C.c_int, C.c_int, C.c_float, C.c_void_p,
                                      C.c_int, C.c_int, _u8p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_crc.restype = C.c_uint32
        L.orc_crc.argtypes = [_u8p, C.c_int, C.c_uint32, C.c_int]
        L.orc_rm_k0.argtypes = [C.c_int, C.c_int, C.c_int]
        L.orc_rm_index.argtypes = [C.c_int] * 6
        L.orc_interleave_src.argtypes = [C.c_int, C.c_int, C.c_int]
        L.orc_gen_rm_llr.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_uint64, C.c_uint64, C.c_int,
                                     _f32p, _i32p, _i32p, _i32p, _i32p, C.c_int, _f32p, C.c_void_p]
        L.orc_derate_match.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _f32p, C.c_int,
                                       _i32p, _i32p, _i32p, _i32p, _f32p]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleCode:
    """A lifted code in the oracle: base matrix (V, -1 empty) and Z."""

    def __init__(self, base: np.ndarray, z: int):
        base = np.ascontiguousarray(base, dtype=np.int32)
        self.rows, self.cols = base.shape
        self.z = int(z)
        self.n_bp = self.cols * self.z
        self.n_bytes = (self.n_bp + 7) // 8
        self.base = base
        self._h = lib().orc_code_new(base, self.rows, self.cols, self.z)
        if not self._h:
            raise ValueError("bad base matrix")
        self.n_edges = lib().orc_code_edges(self._h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_code_free(self._h)
            self._h = None

    def minsum_f32(self, llr, n_iter, alpha=0.75, early_stop=False, want_app=False, threads=1):
        llr = np.ascontiguousarray(llr, dtype=np.float32).reshape(-1, self.n_bp)
        n = llr.shape[0]
        packed = np.zeros((n, self.n_bytes), np.uint8)
        app = np.zeros((n, self.n_bp), np.float32) if want_app else None
        iters = np.zeros(n, np.int32)
        rc = lib().orc_minsum_f32(self._h, llr, n, int(n_iter), float(alpha), int(early_stop),
                                  packed, _ptr(app), _ptr(iters), int(threads))
        if rc:
            raise RuntimeError(f"orc_minsum_f32 rc={rc}")
        return packed, app, iters

    def layered_f32(self, llr, n_iter, alpha=0.75, w=None, early_stop=False, want_app=False, threads=1):
        """Layered-schedule min-sum (w: [T, E] weights or None for alpha)."""
        llr = np.ascontiguousarray(llr, dtype=np.float32).reshape(-1, self.n_bp)
        n = llr.shape[0]
        packed = np.zeros((n, self.n_bytes), np.uint8)
        app = np.zeros((n, self.n_bp), np.float32) if want_app else None
        iters = np.zeros(n, np.int32)
        wa = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
        rc = lib().orc_layered_f32(self._h, llr, n, int(n_iter), float(alpha), _ptr(wa),
                                   0 if wa is None else wa.shape[0], int(early_stop), packed, _ptr(app),
                                   _ptr(iters), int(threads))
        if rc:
            raise RuntimeError(f"orc_layered_f32 rc={rc}")
        return packed, app, iters

    def minsum_f64(self, llr, n_iter, alpha=0.75, early_stop=False):
        llr = np.ascontiguousarray(llr, dtype=np.float64).reshape(-1, self.n_bp)
        n = llr.shape[0]
        packed = np.zeros((n, self.n_bytes), np.uint8)
        app = np.zeros((n, self.n_bp), np.float64)
        iters = np.zeros(n, np.int32)
        rc = lib().orc_minsum_f64(self._h, llr, n, int(n_iter), float(alpha), int(early_stop),
                                  packed, _ptr(app), _ptr(iters))
        if rc:
            raise RuntimeError(f"orc_minsum_f64 rc={rc}")
        return packed, app, iters

    def syndrome_weight(self, packed_cw) -> int:
        return lib().orc_syndrome_weight(self._h, np.ascontiguousarray(packed_cw, np.uint8))

    def encode(self, kb, info_bits):
        out = np.zeros(self.n_bytes, np.uint8)
        rc = lib().orc_encode(self._h, int(kb), np.ascontiguousarray(info_bits, np.uint8), out)
        if rc:
            raise RuntimeError(f"orc_encode rc={rc}")
        return out

    def gen_llr(self, kb, seed, cw_base, sigma, n_punct_cols):
        sigma = np.ascontiguousarray(np.atleast_1d(sigma), np.float32)
        n = sigma.shape[0]
        llr = np.zeros((n, self.n_bp), np.float32)
        cw = np.zeros((n, self.n_bytes), np.uint8)
        rc = lib().orc_gen_llr(self._h, int(kb), int(seed), int(cw_base), n, sigma,
                               int(n_punct_cols), llr, _ptr(cw))
        if rc:
            raise RuntimeError(f"orc_gen_llr rc={rc}")
        return llr, cw

    def wms_loss_grad(self, llr, cw_packed, n_iter, w, want_grad=True, layered=False, f32_forward=False):
        """Loss, dloss/dw and final posterior of the weighted decoder (f64;
        layered: the row-sequential schedule, f32_forward: its forward in the
        decoder's fp32 rounding)."""
        llr = np.ascontiguousarray(llr, np.float32).reshape(-1, self.n_bp)
        n = llr.shape[0]
        w = np.ascontiguousarray(w, np.float64).reshape(n_iter, self.n_edges)
        grad = np.zeros_like(w) if want_grad else None
        app = np.zeros((n, self.n_bp), np.float64)
        cw = np.ascontiguousarray(cw_packed, np.uint8)
        if layered:
            loss = lib().orc_wms_layered_loss_grad(self._h, llr, cw, n, int(n_iter), w, _ptr(grad), _ptr(app),
                                                   int(f32_forward))
        else:
            loss = lib().orc_wms_loss_grad_f64(self._h, llr, cw, n, int(n_iter), w, _ptr(grad), _ptr(app))
        return loss, grad, app

    def wms_decode_f32(self, llr, n_iter, w, early_stop=False, want_app=False):
        llr = np.ascontiguousarray(llr, dtype=np.float32).reshape(-1, self.n_bp)
        w = np.ascontiguousarray(w, np.float32).reshape(-1, self.n_edges)
        n = llr.shape[0]
        packed = np.zeros((n, self.n_bytes), np.uint8)
        app = np.zeros((n, self.n_bp), np.float32) if want_app else None
        iters = np.zeros(n, np.int32)
        rc = lib().orc_wms_decode_f32(self._h, llr, n, int(n_iter), w, w.shape[0],
                                      int(early_stop), packed, _ptr(app), _ptr(iters))
        if rc:
            raise RuntimeError(f"orc_wms_decode_f32 rc={rc}")
        return packed, app, iters


CRC24A, CRC24B, CRC16 = (0x864CFB, 24), (0x800063, 24), (0x1021, 16)


def crc(packed, n_bits, poly_len):
    return lib().orc_crc(np.ascontiguousarray(packed, np.uint8), int(n_bits), poly_len[0], poly_len[1])


def rm_k0(bg, z, rv):
    return lib().orc_rm_k0(bg, z, rv)


def rm_index(z, ncb, kb_z, k_prime, k0, k):
    return lib().orc_rm_index(z, ncb, kb_z, k_prime, k0, k)


def interleave_src(e, qm, p):
    """e index of the bit sent at position p (TS 38.212 5.4.2.2)."""
    return lib().orc_interleave_src(int(e), int(qm), int(p))


def gen_rm_llr(oc, kb, bg, seed, cw_base, sigma, k_prime, e, rv, qm=1):
    sigma = np.ascontiguousarray(np.atleast_1d(sigma), np.float32)
    n = sigma.shape[0]
    kp = np.ascontiguousarray(np.broadcast_to(k_prime, (n,)), np.int32)
    ee = np.ascontiguousarray(np.broadcast_to(e, (n,)), np.int32)
    rr = np.ascontiguousarray(np.broadcast_to(rv, (n,)), np.int32)
    qq = np.ascontiguousarray(np.broadcast_to(qm, (n,)), np.int32)
    stride = int(ee.max())
    llr_e = np.zeros((n, stride), np.float32)
    cw = np.zeros((n, oc.n_bytes), np.uint8)
    rc = lib().orc_gen_rm_llr(oc._h, kb, bg, int(seed), int(cw_base), n, sigma, kp, ee, rr, qq, stride,
                              llr_e, _ptr(cw))
    if rc:
        raise RuntimeError(f"orc_gen_rm_llr rc={rc}")
    return llr_e, cw


def derate_match(oc, kb, bg, llr_e, k_prime, e, rv, qm=1):
    llr_e = np.ascontiguousarray(llr_e, np.float32)
    n, stride = llr_e.shape
    kp = np.ascontiguousarray(np.broadcast_to(k_prime, (n,)), np.int32)
    ee = np.ascontiguousarray(np.broadcast_to(e, (n,)), np.int32)
    rr = np.ascontiguousarray(np.broadcast_to(rv, (n,)), np.int32)
    qq = np.ascontiguousarray(np.broadcast_to(qm, (n,)), np.int32)
    out = np.zeros((n, oc.n_bp), np.float32)
    rc = lib().orc_derate_match(oc._h, kb, bg, n, llr_e, stride, kp, ee, rr, qq, out)
    if rc:
        raise RuntimeError(f"orc_derate_match rc={rc}")
    return out


def philox4x32(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32(c, k, o)
    return list(o)


class RefEmu:
    """The reference's own decoder source run on the CPU (oracle/_ref)."""

    KIND = {(46, 68): "bg1", (42, 52): "bg2", (12, 24): "wifi"}

    def __init__(self, base: np.ndarray, z: int):
        kind = self.KIND[tuple(base.shape)]
        path = os.path.join(REF_DIR, f"libref_{kind}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.L = C.CDLL(path)
        self.L.ref_init_code.argtypes = [_i32p, C.c_int, C.c_int, C.c_int]
        self.L.ref_decode.argtypes = [_f32p, C.c_int, C.c_int, _u8p, C.c_void_p]
        self.L.ref_setup_ldpc.argtypes = [C.c_int, C.c_float, C.c_int, _i32p]
        self.L.ref_transmit_llr.argtypes = [C.c_int, C.c_float, C.c_int, C.c_float, C.c_uint,
                                            _f32p, _i32p]
        self.L.ref_constant_image.argtypes = [C.c_void_p, C.c_int]
        h = np.ascontiguousarray(base, np.int32).copy()
        h[h >= 0] %= int(z)
        self.rows, self.cols = h.shape
        self.z = int(z)
        self.n_bp = self.cols * self.z
        self.n_bytes = (self.n_bp + 7) // 8
        rc = self.L.ref_init_code(h, self.rows, self.cols, self.z)
        if rc:
            raise RuntimeError(f"ref_init_code rc={rc}")

    @staticmethod
    def available(kind="bg1") -> bool:
        return os.path.exists(os.path.join(REF_DIR, f"libref_{kind}.so"))

    def decode(self, llr, n_iter, want_app=False, chunk=16):
        llr = np.ascontiguousarray(llr, dtype=np.float32).reshape(-1, self.n_bp)
        n = llr.shape[0]
        packed = np.zeros((n, self.n_bytes), np.uint8)
        app = np.zeros((n, self.n_bp), np.float32) if want_app else None
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            pk = np.zeros((e - s, self.n_bytes), np.uint8)
            ap = np.zeros((e - s, self.n_bp), np.float32) if want_app else None
            rc = self.L.ref_decode(np.ascontiguousarray(llr[s:e]), e - s, int(n_iter), pk, _ptr(ap))
            if rc:
                raise RuntimeError(f"ref_decode rc={rc}")
            packed[s:e] = pk
            if want_app:
                app[s:e] = ap
        return packed, app

    def constant_image(self) -> bytes:
        """The constant memory the reference's setup writes for this code
        (one codeword per block column), as the bytes of its kernels' arrays."""
        buf = (C.c_ubyte * (1 << 16))()
        n = self.L.ref_constant_image(C.cast(buf, C.c_void_p), len(buf))
        if n <= 0:
            raise RuntimeError(f"ref_constant_image rc={n}")
        return bytes(buf[:n])

    def setup_ldpc(self, A, rate, n_iter):
        out = np.zeros(12, np.int32)
        self.L.ref_setup_ldpc(int(A), float(rate), int(n_iter), out)
        keys = ["A", "bg_index", "Z", "K", "N", "H_rows", "H_cols", "n_nz_in_row", "n_nz_in_col",
                "n_iterations", "N_before_puncture", "H00"]
        return dict(zip(keys, out.tolist()))

    def transmit_llr(self, A, rate, n_cw, ebn0_db, seed, K, n_bp):
        llr = np.zeros((n_cw, n_bp), np.float32)
        info = np.zeros((n_cw, K), np.int32)
        rc = self.L.ref_transmit_llr(int(A), float(rate), int(n_cw), float(ebn0_db), int(seed), llr, info)
        if rc:
            raise RuntimeError(f"ref_transmit_llr rc={rc}")
        return llr, info


class RefGPU:
    """The reference's own CUDA kernels (src/ldpc_kernels.cu compiled for the
    GPU with nvcc's default flags into oracle/_ref/ref_kernels_bg1.cubin) run
    on the GPU in its launch sequence by oracle/ref_gpu_harness.cpp, for its
    own configuration: BG1, Z = 384.  Exists only where the reference tree was
    present when oracle/_ref was built (the cubin and the constant image are
    prebuilt there and travel with the repository copy)."""

    ROWS, COLS, Z, MAX_ROW_DEG = 46, 68, 384, 19

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_GPU_CUBIN) and os.path.exists(REF_GPU_CONST)

    def __init__(self):
        if not os.path.exists(REF_GPU_LIB):
            subprocess.run(["make", "-C", HERE, os.path.join("_build", "libref_gpu.so")], check=True,
                           stdout=subprocess.DEVNULL)
        self.L = C.CDLL(REF_GPU_LIB)
        self.L.refgpu_decode.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                         _f32p, C.c_int, C.c_int, _u8p, C.c_void_p]
        self.L.refgpu_time.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       _f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float)]
        self.L.refgpu_latency.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          _f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float),
                                          C.POINTER(C.c_float)]
        with open(REF_GPU_CONST, "rb") as f:
            self.image = f.read()
        self.n_bp = self.COLS * self.Z

    def decode(self, llr, n_iter, want_app=False):
        llr = np.ascontiguousarray(llr, dtype=np.float32).reshape(-1, self.n_bp)
        n = llr.shape[0]
        packed = np.zeros((n, self.n_bp // 8), np.uint8)
        app = np.zeros((n, self.n_bp), np.float32) if want_app else None
        rc = self.L.refgpu_decode(REF_GPU_CUBIN.encode(), self.image, len(self.image), self.ROWS, self.COLS,
                                  self.Z, self.MAX_ROW_DEG, llr, n, int(n_iter), packed, _ptr(app))
        if rc:
            raise RuntimeError(f"refgpu_decode rc={rc}")
        return packed, app

    def time_ms(self, llr, n_iter, warmup=3, reps=10) -> float:
        """Mean device milliseconds of one decode of these LLRs (at most 446
        codewords, the reference's per-stream limit), LLRs resident."""
        llr = np.ascontiguousarray(llr, dtype=np.float32).reshape(-1, self.n_bp)
        ms = C.c_float()
        rc = self.L.refgpu_time(REF_GPU_CUBIN.encode(), self.image, len(self.image), self.ROWS, self.COLS, self.Z,
                                self.MAX_ROW_DEG, llr, llr.shape[0], int(n_iter), int(warmup), int(reps),
                                C.byref(ms))
        if rc:
            raise RuntimeError(f"refgpu_time rc={rc}")
        return ms.value

    def latency_us(self, llr, n_iter, warmup=5, reps=50):
        """The reference testbench's latency (test_latency): host-clock
        microseconds of one call -- H2D from pinned memory, the kernels, D2H
        of the packed bits, synchronize -- as (best, median)."""
        llr = np.ascontiguousarray(llr, dtype=np.float32).reshape(-1, self.n_bp)
        best, med = C.c_float(), C.c_float()
        rc = self.L.refgpu_latency(REF_GPU_CUBIN.encode(), self.image, len(self.image), self.ROWS, self.COLS,
                                   self.Z, self.MAX_ROW_DEG, llr, llr.shape[0], int(n_iter), int(warmup), int(reps),
                                   C.byref(best), C.byref(med))
        if rc:
            raise RuntimeError(f"refgpu_latency rc={rc}")
        return best.value, med.value


def set_fma_dt(on: bool) -> None:
    """orc_minsum_f32 computes dt = R_new - R_old as one fused multiply-add
    (on) or with the source's two roundings (off, the default)."""
    lib().orc_set_fma_dt(1 if on else 0)


# ---- code-block segmentation (3GPP TS 38.212 5.2.2), restated -----------------------
LIFTING_SIZES = sorted({a << j for a in (2, 3, 5, 7, 9, 11, 13, 15) for j in range(8) if a << j <= 384})


def segment_info(B: int, bg: int) -> dict:
    """C, L, K', K, Zc, Kb and filler count for a B-bit transport block (its
    CRC included); None when B + C*L does not divide by C."""
    kcb = 8448 if bg == 1 else 3840
    if B <= kcb:
        L, Cn = 0, 1
    else:
        L = 24
        Cn = -(-B // (kcb - L))
    if (B + Cn * L) % Cn:
        return None
    kp = (B + Cn * L) // Cn
    if bg == 1:
        kb = 22
    else:
        kb = 10 if B > 640 else 9 if B > 560 else 8 if B > 192 else 6
    zc = min(z for z in LIFTING_SIZES if kb * z >= kp)
    k = (22 if bg == 1 else 10) * zc
    return {"B": B, "C": Cn, "L": L, "k_prime": kp, "k": k, "zc": zc, "kb": kb, "filler": k - kp, "bg": bg}


def cb_segment(tb_bits: np.ndarray, info: dict) -> np.ndarray:
    """[C, K'] bits of the code blocks: consecutive TB bits, then CRC24B (MSB
    first) when C > 1."""
    Cn, L, kp = info["C"], info["L"], info["k_prime"]
    d = kp - L
    out = np.zeros((Cn, kp), np.uint8)
    for r in range(Cn):
        out[r, :d] = tb_bits[r * d:(r + 1) * d]
        if L:
            rem = crc(np.packbits(out[r, :d], bitorder="little"), d, CRC24B)
            out[r, d:] = [(rem >> (L - 1 - i)) & 1 for i in range(L)]
    return out
