"""ctypes binding of libpermgpu.so (the C ABI declared in include/permgpu.h).

The library is loaded from this package directory.  There is no CPU
fallback: if the shared object is missing or no CUDA device is usable, the
calls raise instead of computing anything on the host.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libpermgpu.so"

PG_OK = 0
PG_EINVAL = 1
PG_ERANGE = 2
PG_ECUDA = 3
PG_ENOMEM = 4
PG_EABORT = 5
PG_ENODEV = 6
PG_EOVERFLOW = 7
PG_EINTERNAL = 8

STATUS_NAMES = {
    PG_OK: "PG_OK", PG_EINVAL: "PG_EINVAL", PG_ERANGE: "PG_ERANGE",
    PG_ECUDA: "PG_ECUDA", PG_ENOMEM: "PG_ENOMEM", PG_EABORT: "PG_EABORT",
    PG_ENODEV: "PG_ENODEV", PG_EOVERFLOW: "PG_EOVERFLOW",
    PG_EINTERNAL: "PG_EINTERNAL",
}

# Every symbol the header declares, with its ctypes signature.
_c_i64p = ctypes.POINTER(ctypes.c_int64)
_c_u64p = ctypes.POINTER(ctypes.c_uint64)
_c_u32p = ctypes.POINTER(ctypes.c_uint32)
_c_u8p = ctypes.POINTER(ctypes.c_uint8)
_c_f64p = ctypes.POINTER(ctypes.c_double)
_c_i32p = ctypes.POINTER(ctypes.c_int32)
_c_intp = ctypes.POINTER(ctypes.c_int)

SIGNATURES = {
    "pg_version": ([], ctypes.c_int),
    "pg_cuda_runtime_available": ([], ctypes.c_int),
    "pg_last_error": ([], ctypes.c_char_p),
    "pg_device_info": ([_c_intp, _c_intp, _c_intp], ctypes.c_int),
    "pg_abort": ([], None),
    "pg_clear_abort": ([], None),
    "pg_residues": ([_c_i64p, ctypes.c_int, _c_u64p, ctypes.c_int, _c_u64p], ctypes.c_int),
    "pg_residues_partial": ([_c_i64p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, _c_u64p,
                             ctypes.c_int, _c_u64p], ctypes.c_int),
    "pg_schur_residues": ([ctypes.c_int, _c_u64p, _c_u64p, ctypes.c_int, _c_u64p], ctypes.c_int),
    "pg_schur_residues_method": ([ctypes.c_int, _c_u64p, _c_u64p, ctypes.c_int, ctypes.c_int,
                                  _c_u64p], ctypes.c_int),
    "pg_necklace_orbit_stats": ([ctypes.c_int, _c_u64p, _c_u64p], ctypes.c_int),
    "pg_glynn_f64_fwd_bwd": ([_c_f64p, ctypes.c_int, ctypes.c_int, _c_f64p, _c_f64p, _c_f64p],
                             ctypes.c_int),
    "pg_glynn_c64": ([_c_f64p, _c_f64p, ctypes.c_int, ctypes.c_int, _c_f64p, _c_f64p, _c_f64p],
                     ctypes.c_int),
    "pg_batch_residues": ([_c_i64p, _c_i64p, _c_i32p, ctypes.c_int, _c_u64p, _c_i32p, _c_u64p],
                          ctypes.c_int),
    "pg_permanent_mod3": ([_c_i64p, ctypes.c_int, _c_intp], ctypes.c_int),
    "pg_permanent_mod3_cols": ([_c_u64p, _c_u64p, ctypes.c_int, _c_intp], ctypes.c_int),
    "pg_affine_residues": ([_c_i64p, _c_i64p, ctypes.c_int, _c_u64p, ctypes.c_int, _c_u64p],
                           ctypes.c_int),
    "pg_affine_residues_partial": ([_c_i64p, _c_i64p, ctypes.c_int, ctypes.c_uint64,
                                    ctypes.c_uint64, _c_u64p, ctypes.c_int, _c_u64p],
                                   ctypes.c_int),
    "pg_binary_residues": ([_c_u8p, ctypes.c_int, _c_u64p, ctypes.c_int, _c_u64p], ctypes.c_int),
    "pg_exact_permanent": ([_c_i64p, ctypes.c_int, _c_u32p, ctypes.c_int], ctypes.c_int),
    "pg_exact_supported": ([_c_i64p, ctypes.c_int], ctypes.c_int),
    "pg_exact_plan_create": ([_c_i64p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "pg_exact_plan_launch": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "pg_exact_plan_result": ([ctypes.c_void_p, ctypes.c_void_p, _c_u32p, ctypes.c_int], ctypes.c_int),
    "pg_exact_plan_info": ([ctypes.c_void_p, _c_intp, _c_intp, _c_u64p, _c_u64p, _c_u64p], ctypes.c_int),
    "pg_exact_plan_destroy": ([ctypes.c_void_p], None),
    "pg_exact_plan_float_rows": ([ctypes.c_void_p], ctypes.c_int),
    "pg_exact_plan_bit_planes": ([ctypes.c_void_p], ctypes.c_int),
    "pg_probe_int_throughput": ([ctypes.c_int, ctypes.c_int, _c_f64p], ctypes.c_int),
    "pg_batch_plan_create": ([_c_i64p, _c_i64p, _c_i32p, ctypes.c_int, ctypes.c_void_p,
                              ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "pg_batch_plan_launch": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "pg_batch_plan_result": ([ctypes.c_void_p, ctypes.c_void_p, _c_u32p, ctypes.c_int], ctypes.c_int),
    "pg_batch_plan_info": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32), _c_intp, _c_u64p,
                            _c_intp], ctypes.c_int),
    "pg_batch_plan_destroy": ([ctypes.c_void_p], None),
    "pg_batch_exact": ([_c_i64p, _c_i64p, _c_i32p, ctypes.c_int, _c_u32p, ctypes.c_int], ctypes.c_int),
    "pg_exact_permanent_noalloc": ([_c_i64p, ctypes.c_int, _c_u32p, ctypes.c_int, ctypes.c_void_p],
                                   ctypes.c_int),
    "pg_exact_partial": ([_c_i64p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, _c_i64p,
                          ctypes.c_int, _c_intp], ctypes.c_int),
    "pg_glynn_c64_dev": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "pg_glynn_window": ([_c_f64p, _c_f64p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                         _c_f64p, _c_f64p, _c_f64p], ctypes.c_int),
    "pg_glynn_f64_dev": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
}


class BatchTune(ctypes.Structure):
    """pg_batch_tune: fields <= 0 select the library defaults."""
    _fields_ = [("lane_log_states", ctypes.c_int), ("chunk_log_len", ctypes.c_int),
                ("blocks_per_sm", ctypes.c_int)]

_lib = None
_lock = threading.Lock()


class PermGpuError(RuntimeError):
    """A libpermgpu call returned a non-zero pg_status."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


def load(path: str | Path | None = None):
    """Load (once) and return the ctypes library handle."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise ImportError(
                f"{p} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                "or `python rivin-perm_gb300/permgpu/_build.py`")
        lib = ctypes.CDLL(str(p))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        if path is None:
            _lib = lib
        return lib


def check(status: int) -> None:
    if status != PG_OK:
        msg = load().pg_last_error()
        raise PermGpuError(status, msg.decode() if msg else "")


def cuda_available() -> bool:
    try:
        return bool(load().pg_cuda_runtime_available())
    except (ImportError, OSError):
        return False


def ptr(arr: np.ndarray, ctype):
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


# --- thin typed wrappers ---------------------------------------------------

def residues(matrix: np.ndarray, moduli) -> list[int]:
    """per(matrix) mod m for each m (matrix: int64 n x n, C order)."""
    a = np.ascontiguousarray(matrix, dtype=np.int64)
    n = a.shape[0] if a.ndim == 2 else 0
    mods = np.ascontiguousarray(np.asarray(list(moduli), dtype=np.uint64))
    out = np.zeros(len(mods), dtype=np.uint64)
    check(load().pg_residues(ptr(a, ctypes.c_int64), n, ptr(mods, ctypes.c_uint64),
                             len(mods), ptr(out, ctypes.c_uint64)))
    return [int(x) for x in out]


SCHUR_METHODS = {"auto": 0, "glynn": 1, "necklace": 2}


def schur_residues(n: int, primes, omegas, method: str = "auto") -> list[int]:
    """perm(S_n) mod each prime; method "auto" | "glynn" | "necklace"."""
    if method not in SCHUR_METHODS:
        raise ValueError(f"unknown Schur method {method!r}")
    ps = np.ascontiguousarray(np.asarray(list(primes), dtype=np.uint64))
    ws = np.ascontiguousarray(np.asarray(list(omegas), dtype=np.uint64))
    out = np.zeros(len(ps), dtype=np.uint64)
    check(load().pg_schur_residues_method(int(n), ptr(ps, ctypes.c_uint64),
                                          ptr(ws, ctypes.c_uint64), len(ps),
                                          SCHUR_METHODS[method], ptr(out, ctypes.c_uint64)))
    return [int(x) for x in out]


def necklace_orbit_stats(n: int) -> tuple[int, int]:
    """(representatives, covered sign words) of the necklace quotient for an
    odd prime order 3 <= n < 64 (host only)."""
    reps, words = ctypes.c_uint64(), ctypes.c_uint64()
    st = load().pg_necklace_orbit_stats(int(n), ctypes.byref(reps), ctypes.byref(words))
    if st == PG_ERANGE:
        raise ValueError(load().pg_last_error().decode())
    check(st)
    return int(reps.value), int(words.value)


def glynn_f64_fwd_bwd(matrices, want_grad: bool = True):
    """(per[batch], grad[batch][n][n] or None, abs_sum[batch]) for a batch of
    real matrices through the host-pointer C entry point."""
    a = np.ascontiguousarray(matrices, dtype=np.float64)
    batch, n = a.shape[0], a.shape[1]
    per = np.zeros(batch, dtype=np.float64)
    grad = np.zeros((batch, n, n), dtype=np.float64) if want_grad else None
    abs_sum = np.zeros(batch, dtype=np.float64)
    check(load().pg_glynn_f64_fwd_bwd(ptr(a, ctypes.c_double), batch, n,
                                      ptr(per, ctypes.c_double),
                                      ptr(grad, ctypes.c_double) if want_grad else None,
                                      ptr(abs_sum, ctypes.c_double)))
    return per, grad, abs_sum


def glynn_c64(matrices):
    """(per[batch] complex128, abs_sum[batch]) for a batch of complex
    matrices through the host-pointer C entry point."""
    a = np.asarray(matrices, dtype=np.complex128)
    re = np.ascontiguousarray(a.real)
    im = np.ascontiguousarray(a.imag)
    batch, n = a.shape[0], a.shape[1]
    per_re = np.zeros(batch, dtype=np.float64)
    per_im = np.zeros(batch, dtype=np.float64)
    abs_sum = np.zeros(batch, dtype=np.float64)
    check(load().pg_glynn_c64(ptr(re, ctypes.c_double), ptr(im, ctypes.c_double), batch, n,
                              ptr(per_re, ctypes.c_double), ptr(per_im, ctypes.c_double),
                              ptr(abs_sum, ctypes.c_double)))
    return per_re + 1j * per_im, abs_sum


def batch_residues(matrices, moduli_lists) -> list[list[int]]:
    """[[per(A_m) mod q for q in moduli_lists[m]] for each matrix A_m]."""
    mats = [np.ascontiguousarray(m, dtype=np.int64) for m in matrices]
    orders = np.array([m.shape[0] if m.ndim == 2 else 0 for m in mats], dtype=np.int32)
    offsets = np.zeros(len(mats), dtype=np.int64)
    if len(mats) > 1:
        offsets[1:] = np.cumsum([m.size for m in mats])[:-1]
    flat = np.ascontiguousarray(np.concatenate([m.ravel() for m in mats]) if mats else
                                np.zeros(1, np.int64), dtype=np.int64)
    if flat.size == 0:
        flat = np.zeros(1, np.int64)
    mods = np.ascontiguousarray(np.array([int(q) for ms in moduli_lists for q in ms] or [1],
                                         dtype=np.uint64))
    moff = np.zeros(len(mats) + 1, dtype=np.int32)
    moff[1:] = np.cumsum([len(ms) for ms in moduli_lists])
    out = np.zeros(max(1, int(moff[-1])), dtype=np.uint64)
    check(load().pg_batch_residues(ptr(flat, ctypes.c_int64), ptr(offsets, ctypes.c_int64),
                                   ptr(orders, ctypes.c_int32), len(mats),
                                   ptr(mods, ctypes.c_uint64), ptr(moff, ctypes.c_int32),
                                   ptr(out, ctypes.c_uint64)))
    return [[int(out[t]) for t in range(moff[m], moff[m + 1])] for m in range(len(mats))]


def permanent_mod3(matrix) -> int:
    """per(A) mod 3 for an int64 matrix of order < 64."""
    a = np.ascontiguousarray(matrix, dtype=np.int64)
    n = a.shape[0] if a.ndim == 2 else 0
    out = ctypes.c_int()
    check(load().pg_permanent_mod3(ptr(a, ctypes.c_int64), n, ctypes.byref(out)))
    return int(out.value)


def permanent_mod3_cols(col_mags, col_sgns, n: int) -> int:
    m = np.ascontiguousarray(np.asarray(col_mags, dtype=np.uint64))
    s = np.ascontiguousarray(np.asarray(col_sgns, dtype=np.uint64))
    out = ctypes.c_int()
    check(load().pg_permanent_mod3_cols(ptr(m, ctypes.c_uint64), ptr(s, ctypes.c_uint64),
                                        int(n), ctypes.byref(out)))
    return int(out.value)


def affine_residues(constant, linear, moduli) -> list[list[int]]:
    """[coefficients of per(C + x L) mod m for m in moduli] (odd m < 2^30,
    int64 entries, order <= 63)."""
    c = np.ascontiguousarray(constant, dtype=np.int64)
    l = np.ascontiguousarray(linear, dtype=np.int64)
    n = c.shape[0] if c.ndim == 2 else 0
    mods = np.ascontiguousarray(np.asarray(list(moduli), dtype=np.uint64))
    out = np.zeros((len(mods), n + 1), dtype=np.uint64)
    check(load().pg_affine_residues(ptr(c, ctypes.c_int64), ptr(l, ctypes.c_int64), n,
                                    ptr(mods, ctypes.c_uint64), len(mods),
                                    ptr(out, ctypes.c_uint64)))
    return [[int(x) for x in row] for row in out]


def affine_residues_partial(constant, linear, lo: int, hi: int, moduli) -> list[list[int]]:
    """[coefficients of the unscaled Glynn sum of per(C + x L) over Gray
    states [lo, hi) mod m for m in moduli] (pg_affine_residues_partial)."""
    c = np.ascontiguousarray(constant, dtype=np.int64)
    l = np.ascontiguousarray(linear, dtype=np.int64)
    n = c.shape[0]
    mods = np.ascontiguousarray(np.asarray(list(moduli), dtype=np.uint64))
    out = np.zeros((len(mods), n + 1), dtype=np.uint64)
    check(load().pg_affine_residues_partial(ptr(c, ctypes.c_int64), ptr(l, ctypes.c_int64), n,
                                            ctypes.c_uint64(lo), ctypes.c_uint64(hi),
                                            ptr(mods, ctypes.c_uint64), len(mods),
                                            ptr(out, ctypes.c_uint64)))
    return [[int(x) for x in row] for row in out]


def binary_residues(matrix: np.ndarray, primes) -> list[int]:
    a = np.ascontiguousarray(matrix, dtype=np.uint8)
    n = a.shape[0] if a.ndim == 2 else 0
    ps = np.ascontiguousarray(np.asarray(list(primes), dtype=np.uint64))
    out = np.zeros(len(ps), dtype=np.uint64)
    check(load().pg_binary_residues(ptr(a, ctypes.c_uint8), n, ptr(ps, ctypes.c_uint64),
                                    len(ps), ptr(out, ctypes.c_uint64)))
    return [int(x) for x in out]


def limbs_to_int(words: np.ndarray) -> int:
    """Two's-complement little-endian uint32 words -> Python int."""
    v = 0
    for i, w in enumerate(words.tolist()):
        v |= int(w) << (32 * i)
    bits = 32 * len(words)
    if v >> (bits - 1):
        v -= 1 << bits
    return v


def exact_supported(matrix: np.ndarray) -> bool:
    a = np.ascontiguousarray(matrix, dtype=np.int64)
    return bool(load().pg_exact_supported(ptr(a, ctypes.c_int64), a.shape[0]))


def exact_limbs(matrix: np.ndarray) -> int:
    """Output words that hold any value within the row-sum bound."""
    bits = 0.0
    for row in np.abs(np.asarray(matrix, dtype=np.float64)):
        bits += float(np.log2(max(1.0, float(row.sum()))))
    return int(bits + 2) // 32 + 2


def exact_permanent(matrix: np.ndarray, limbs: int) -> int:
    a = np.ascontiguousarray(matrix, dtype=np.int64)
    out = np.zeros(limbs, dtype=np.uint32)
    check(load().pg_exact_permanent(ptr(a, ctypes.c_int64), a.shape[0],
                                    ptr(out, ctypes.c_uint32), limbs))
    return limbs_to_int(out)


class ExactPlan:
    """Device-resident exact evaluation of one matrix (pg_exact_plan_*)."""

    def __init__(self, matrix: np.ndarray):
        a = np.ascontiguousarray(matrix, dtype=np.int64)
        self.n = a.shape[0]
        self.limbs = exact_limbs(a)
        h = ctypes.c_void_p()
        check(load().pg_exact_plan_create(ptr(a, ctypes.c_int64), self.n, ctypes.byref(h)))
        self._h = h
        g, w = ctypes.c_int(), ctypes.c_int()
        st, imul, wide = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(load().pg_exact_plan_info(h, ctypes.byref(g), ctypes.byref(w), ctypes.byref(st),
                                        ctypes.byref(imul), ctypes.byref(wide)))
        self.group, self.words, self.states = g.value, w.value, st.value
        self.imul_per_state, self.imad_wide_per_state = imul.value, wide.value
        self.float_rows = int(load().pg_exact_plan_float_rows(h))
        self.bit_planes = int(load().pg_exact_plan_bit_planes(h))

    def launch(self, stream: int | None = None) -> None:
        check(load().pg_exact_plan_launch(self._h, ctypes.c_void_p(stream or 0)))

    def result(self, stream: int | None = None) -> int:
        out = np.zeros(self.limbs, dtype=np.uint32)
        check(load().pg_exact_plan_result(self._h, ctypes.c_void_p(stream or 0),
                                          ptr(out, ctypes.c_uint32), self.limbs))
        return limbs_to_int(out)

    def close(self) -> None:
        if self._h:
            load().pg_exact_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pack_batch(matrices):
    """(A_packed int64, offsets int64, orders int32) for a list of square
    integer matrices."""
    orders = np.array([np.asarray(m).shape[0] if np.asarray(m).ndim == 2 else 0
                       for m in matrices], dtype=np.int32)
    sizes = orders.astype(np.int64) ** 2
    offsets = np.zeros(len(matrices), dtype=np.int64)
    if len(matrices) > 1:
        offsets[1:] = np.cumsum(sizes)[:-1]
    packed = np.zeros(int(sizes.sum()) or 1, dtype=np.int64)
    for m, off, sz in zip(matrices, offsets, sizes):
        if sz:
            packed[off:off + sz] = np.asarray(m, dtype=np.int64).reshape(-1)
    return packed, offsets, orders


def batch_limbs(matrices) -> int:
    return max([exact_limbs(np.asarray(m)) for m in matrices if np.asarray(m).size] or [2])


class BatchPlan:
    """Device-resident batched exact evaluation (pg_batch_plan_*): one
    persistent work-stealing launch per evaluation, replayed from a CUDA
    graph."""

    def __init__(self, matrices, tune: tuple | None = None):
        self.count = len(matrices)
        self.limbs = batch_limbs(matrices)
        packed, offsets, orders = pack_batch(matrices)
        self.orders = orders
        t = BatchTune(*(tune or (0, 0, 0)))
        h = ctypes.c_void_p()
        check(load().pg_batch_plan_create(ptr(packed, ctypes.c_int64), ptr(offsets, ctypes.c_int64),
                                          ptr(orders, ctypes.c_int32), self.count,
                                          ctypes.byref(t), ctypes.byref(h)))
        self._h = h
        nt, nb, st, ext = ctypes.c_uint32(), ctypes.c_int(), ctypes.c_uint64(), ctypes.c_int()
        check(load().pg_batch_plan_info(h, ctypes.byref(nt), ctypes.byref(nb), ctypes.byref(st),
                                        ctypes.byref(ext)))
        self.tasks, self.blocks, self.kernel_states, self.external = nt.value, nb.value, st.value, ext.value

    def launch(self, stream: int | None = None) -> None:
        check(load().pg_batch_plan_launch(self._h, ctypes.c_void_p(stream or 0)))

    def results(self, stream: int | None = None) -> list[int]:
        out = np.zeros(self.count * self.limbs, dtype=np.uint32)
        check(load().pg_batch_plan_result(self._h, ctypes.c_void_p(stream or 0),
                                          ptr(out, ctypes.c_uint32), self.limbs))
        return [limbs_to_int(out[i * self.limbs:(i + 1) * self.limbs]) for i in range(self.count)]

    def close(self) -> None:
        if self._h:
            load().pg_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_exact(matrices) -> list[int]:
    """One-shot host-to-host batched evaluation (pg_batch_exact)."""
    limbs = batch_limbs(matrices)
    packed, offsets, orders = pack_batch(matrices)
    out = np.zeros(len(matrices) * limbs, dtype=np.uint32)
    check(load().pg_batch_exact(ptr(packed, ctypes.c_int64), ptr(offsets, ctypes.c_int64),
                                ptr(orders, ctypes.c_int32), len(matrices),
                                ptr(out, ctypes.c_uint32), limbs))
    return [limbs_to_int(out[i * limbs:(i + 1) * limbs]) for i in range(len(matrices))]


def probe_int_throughput(variant: int, iters: int = 4096) -> float:
    v = ctypes.c_double()
    check(load().pg_probe_int_throughput(int(variant), int(iters), ctypes.byref(v)))
    return v.value
