"""The reference's own CUDA kernels on this GPU — TEST AND MEASUREMENT INFRASTRUCTURE ONLY.

``oracle/build_ref.sh`` compiles the device code of rivin-perm's CUDA tools
(perm_modp_cuda.cu, perm_binary_cuda.cu, perm_parallel_cuda.cu), unmodified,
into cubins under ``oracle/_ref/``.  A cubin holds device code only, so it
runs on any host of the GPU it was built for.  This module loads the cubins
through the CUDA driver API and restates, in Python, the host code around
each kernel: argument checks, matrix normalisation, launch shapes, constant
tables, the reduction passes and the final scaling, following the cited
lines.  It serves two purposes:

* parity: the reference's GPU residues and FP64 values are compared with
  this repository's kernels on the same inputs (tests/test_gpu_reference_cuda.py);
* measurement: ``python oracle/ref_cuda.py`` times the reference's kernels
  on the benchmark workloads on the same GPU as this repository's.

Nothing in the product imports this module.  Device buffers come from
PyTorch, launches go to the caller's (or PyTorch's current) stream.
"""

from __future__ import annotations

import ctypes
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
CUBINS = {"modp": REF_DIR / "perm_modp_cuda.cubin",
          "binary": REF_DIR / "perm_binary_cuda.cubin",
          "parallel": REF_DIR / "perm_parallel_cuda.cubin"}

# kernel names (Itanium mangling of the reference's declarations)
K_RYSER = "_Z21permanent_modp_kernelPKlimmmmPm"            # perm_modp_cuda.cu:229
K_GLYNN = "_Z27permanent_glynn_modp_kernelPKlimmmmPm"      # perm_modp_cuda.cu:328
K_REDUCE = "_Z15reduce_sum_modpPKmPmmm"                     # perm_modp_cuda.cu:706
PM32_ORDERS = (28, 30, 32, 34, 36, 38, 40, 42, 44)          # perm_modp_cuda.cu:870-885
K_F64 = "_Z22permanent_glynn_kernelILb0EEvPKdS1_immPdS2_"  # perm_parallel_cuda.cu:69
K_F64_REDUCE = "_Z13reduce_kernelILb0EEvPKdS1_mPdS2_"      # perm_parallel_cuda.cu:216


def k_pm32(n: int) -> str:                                  # perm_modp_cuda.cu:412
    return f"_Z32permanent_glynn_modp_pm32_kernelILi{n}EEvPKjjjmmmPm"


def available() -> bool:
    return all(p.exists() for p in CUBINS.values())


class DriverError(RuntimeError):
    pass


class _Driver:
    """The few CUDA driver calls needed to load a cubin and launch from it."""

    def __init__(self):
        import torch
        torch.cuda.init()
        torch.empty(1, device="cuda")          # the primary context is current now
        self.cu = ctypes.CDLL("libcuda.so.1")
        cu = self.cu
        vp, u = ctypes.c_void_p, ctypes.c_uint
        sig = {
            "cuInit": [u],
            "cuCtxGetCurrent": [ctypes.POINTER(vp)],
            "cuModuleLoad": [ctypes.POINTER(vp), ctypes.c_char_p],
            "cuModuleGetFunction": [ctypes.POINTER(vp), vp, ctypes.c_char_p],
            "cuModuleGetGlobal_v2": [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_size_t),
                                     vp, ctypes.c_char_p],
            "cuModuleGetFunctionCount": [ctypes.POINTER(u), vp],
            "cuModuleEnumerateFunctions": [ctypes.POINTER(vp), u, vp],
            "cuFuncGetName": [ctypes.POINTER(ctypes.c_char_p), vp],
            "cuMemcpyHtoD_v2": [ctypes.c_uint64, vp, ctypes.c_size_t],
            "cuLaunchKernel": [vp, u, u, u, u, u, u, u, vp, ctypes.POINTER(vp), ctypes.POINTER(vp)],
            "cuGetErrorString": [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)],
        }
        for name, args in sig.items():
            f = getattr(cu, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        self.check(cu.cuInit(0), "cuInit")
        ctx = vp()
        self.check(cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise DriverError("no current CUDA context after PyTorch initialisation")
        self.modules = {}

    def check(self, rc: int, what: str):
        if rc != 0:
            msg = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(msg))
            raise DriverError(f"{what}: CUDA driver error {rc} ({(msg.value or b'').decode()})")

    def module(self, key: str):
        if key not in self.modules:
            path = CUBINS[key]
            if not path.exists():
                raise DriverError(f"{path} not built (oracle/build_ref.sh REFERENCE_DIR)")
            mod = ctypes.c_void_p()
            self.check(self.cu.cuModuleLoad(ctypes.byref(mod), str(path).encode()), f"load {path.name}")
            self.modules[key] = mod
        return self.modules[key]

    def function(self, key: str, name: str):
        f = ctypes.c_void_p()
        self.check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.module(key), name.encode()),
                   f"function {name}")
        return f

    def function_containing(self, key: str, part: str):
        """A kernel found by a substring of its name (names in anonymous
        namespaces carry a per-translation-unit tag)."""
        mod = self.module(key)
        count = ctypes.c_uint()
        self.check(self.cu.cuModuleGetFunctionCount(ctypes.byref(count), mod), "function count")
        funcs = (ctypes.c_void_p * count.value)()
        self.check(self.cu.cuModuleEnumerateFunctions(funcs, count.value, mod), "enumerate functions")
        for f in funcs:
            name = ctypes.c_char_p()
            self.check(self.cu.cuFuncGetName(ctypes.byref(name), f), "function name")
            if part in name.value.decode():
                return ctypes.c_void_p(f), name.value.decode()
        raise DriverError(f"no kernel named *{part}* in {CUBINS[key].name}")

    def set_global(self, key: str, names, data: bytes):
        """Copies `data` into the first of `names` that the module defines
        (synchronous; the caller orders it against its stream)."""
        mod = self.module(key)
        for name in names:
            dptr, size = ctypes.c_uint64(), ctypes.c_size_t()
            if self.cu.cuModuleGetGlobal_v2(ctypes.byref(dptr), ctypes.byref(size), mod,
                                            name.encode()) == 0:
                if size.value < len(data):
                    raise DriverError(f"{name}: {size.value} bytes, {len(data)} given")
                buf = ctypes.create_string_buffer(data, len(data))
                self.check(self.cu.cuMemcpyHtoD_v2(dptr.value, buf, len(data)), f"copy to {name}")
                return
        raise DriverError(f"none of {names} in {CUBINS[key].name}")

    def launch(self, f, grid: int, block: int, smem: int, stream: int, args):
        """args: ctypes scalars in the kernel's parameter order."""
        holders = list(args)
        params = (ctypes.c_void_p * len(holders))(
            *[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p) for h in holders])
        self.check(self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, ctypes.c_void_p(stream),
                                          params, None), "cuLaunchKernel")


_drv = None


def driver() -> _Driver:
    global _drv
    if _drv is None:
        _drv = _Driver()
    return _drv


def _stream(stream):
    import torch
    return (stream or torch.cuda.current_stream()).cuda_stream


def _ptr(t) -> ctypes.c_uint64:
    return ctypes.c_uint64(t.data_ptr())


def _reduce_modp(partial, count: int, p: int, stream: int):
    """perm_modp_cuda.cu:826-838 (and :1213-1232): passes of reduce_sum_modp,
    256 threads, two inputs per thread, until one value is left."""
    import torch
    d = driver()
    f = d.function("modp", K_REDUCE)
    other = torch.empty(count, dtype=torch.int64, device="cuda")
    src, dst, size = partial, other, count
    while size > 1:
        blocks = (size + 511) // 512
        d.launch(f, blocks, 256, 256 * 8, stream,
                 [_ptr(src), _ptr(dst), ctypes.c_uint64(size), ctypes.c_uint64(p)])
        size = blocks
        src, dst = dst, src
    return src


def permanent_modp(matrix, p: int, stream=None, timer=None) -> int:
    """perm_modp_cuda.cu:740-868 (permanent_modp_cuda): Ryser's formula over
    2^n column subsets in Gray order, modulus p < 2^63, 64-bit arithmetic."""
    import torch
    a = np.asarray(matrix, dtype=np.int64)
    n = a.shape[0]
    if not (2 <= n < 64) or p <= 0:
        raise ValueError("n must satisfy 2 <= n < 64 and p > 0")
    num_subsets = 1 << n
    if n >= 30:
        total_threads = 1 << 18
        block_size = (num_subsets + total_threads - 1) // total_threads
    elif n >= 20:
        total_threads = 1 << 14
        block_size = (num_subsets + total_threads - 1) // total_threads
    else:
        total_threads, block_size = num_subsets, 1
    num_blocks = (total_threads + 255) // 256
    norm = torch.from_numpy(np.mod(a, p).astype(np.int64).ravel()).cuda()
    partial = torch.empty(total_threads, dtype=torch.int64, device="cuda")
    s = _stream(stream)
    d = driver()
    if timer:
        timer.start(stream)
    d.launch(d.function("modp", K_RYSER), num_blocks, 256, 0, s,
             [_ptr(norm), ctypes.c_int(n), ctypes.c_uint64(p), ctypes.c_uint64(num_subsets),
              ctypes.c_uint64(block_size), ctypes.c_uint64(total_threads), _ptr(partial)])
    out = _reduce_modp(partial, total_threads, p, s)
    if timer:
        timer.stop(stream)
    r = int(out[:1].cpu().item()) & ((1 << 64) - 1)
    if n & 1:                                    # perm_modp_cuda.cu:846-849
        r = 0 if r == 0 else p - r
    return r


def glynn_modp(matrix, p: int, stream=None, timer=None) -> int:
    """perm_modp_cuda.cu:1119-1262 (permanent_glynn_modp_cuda_internal):
    Glynn's formula, last sign fixed; the pseudo-Mersenne kernel
    permanent_glynn_modp_pm32_kernel<N> for p = 2^32 - c (1 <= c < 2^16) at
    its compiled orders, else the generic 64-bit kernel.  p odd."""
    import torch
    a = np.asarray(matrix, dtype=np.int64)
    n = a.shape[0]
    if n < 2 or n >= 64 or p <= 2 or p % 2 == 0:
        raise ValueError("n must satisfy 2 <= n < 64 and p must be odd")
    num_states = 1 << (n - 1)
    if n >= 28:
        total_threads = 1 << 18
        block_size = (num_states + total_threads - 1) // total_threads
    elif n >= 20:
        total_threads = 1 << 14
        block_size = (num_states + total_threads - 1) // total_threads
    else:
        total_threads, block_size = num_states, 1
    num_blocks = (total_threads + 255) // 256
    gap = (1 << 32) - p
    pm32 = p <= 0xFFFFFFFF and n in PM32_ORDERS and 1 <= gap <= 0xFFFF
    d = driver()
    s = _stream(stream)
    partial = torch.empty(total_threads, dtype=torch.int64, device="cuda")
    if pm32:
        norm = torch.from_numpy(np.mod(a, p).astype(np.uint32).view(np.int32).ravel()).cuda()
        f = d.function("modp", k_pm32(n))
        args = [_ptr(norm), ctypes.c_uint32(p), ctypes.c_uint32(gap), ctypes.c_uint64(num_states),
                ctypes.c_uint64(block_size), ctypes.c_uint64(total_threads), _ptr(partial)]
    else:
        norm = torch.from_numpy(np.mod(a, p).astype(np.int64).ravel()).cuda()
        f = d.function("modp", K_GLYNN)
        args = [_ptr(norm), ctypes.c_int(n), ctypes.c_uint64(p), ctypes.c_uint64(num_states),
                ctypes.c_uint64(block_size), ctypes.c_uint64(total_threads), _ptr(partial)]
    if timer:
        timer.start(stream)
    d.launch(f, num_blocks, 256, 0, s, args)
    out = _reduce_modp(partial, total_threads, p, s)
    if timer:
        timer.stop(stream)
    r = int(out[:1].cpu().item()) & ((1 << 64) - 1)
    return r * pow((p >> 1) + 1, n - 1, p) % p        # 2^(1-n), perm_modp_cuda.cu:1242-1246


# --- perm_modp_cuda.cu: Schur necklace kernel -----------------------------

NECKLACE_CONFIG = {40: (24, 256, 4), 46: (28, 256, 4)}   # perm_modp_cuda.cu:923-930
NECKLACE_TASK = np.dtype([("word", "<u8"), ("period", "<u4"), ("weight", "<u4")])


def k_necklace(m: int, depth: int) -> str:                    # perm_modp_cuda.cu:618
    return (f"_Z26schur_necklace_pm32_kernelILi{m}ELi{depth}EEvPK18NecklacePrefixTask"
            f"jPKjjjjPjPy")


def necklace_frontier(m: int, depth: int) -> np.ndarray:
    """perm_modp_cuda.cu:91-147 (build_necklace_frontier): FKM prefixes of
    length `depth` of pre-necklaces of length m with weight <= m/2, each with
    its period and weight, the word left-aligned to m bits."""
    tasks = []
    bits = [0] * 64

    def rec(position, period, weight, prefix):
        if position > depth:
            tasks.append((prefix << (m - depth), period, weight))
            return
        copied = bits[position - period]
        if weight + copied <= m // 2:
            bits[position] = copied
            rec(position + 1, period, weight + copied, (prefix << 1) | copied)
        if copied == 0 and weight + 1 <= m // 2:
            bits[position] = 1
            rec(position + 1, position, weight + 1, (prefix << 1) | 1)
    rec(1, 1, 0, 0)
    return np.array(tasks, dtype=NECKLACE_TASK)


_frontiers = {}


def _smallest_primitive_root_prime(n: int) -> int:         # perm_modp_cuda.cu:151-165
    for g in range(2, n):
        v, ok = 1, True
        for _ in range(1, n - 1):
            v = v * g % n
            if v == 1:
                ok = False
                break
        if ok:
            return g
    raise ValueError("no primitive root")


def schur_necklace_modp(n: int, omega: int, p: int, stream=None, timer=None) -> int:
    """perm_modp_cuda.cu:970-1111 (schur_necklace_modp_cuda_internal):
    perm(S_n) mod p for prime n with n - 1 in {40, 46}, p = 2^32 - c
    (1 <= c < 2^16) and omega^n == 1, by the reference's persistent necklace
    kernel over its FKM frontier."""
    import torch
    m = n - 1
    gap = (1 << 32) - p
    if (n < 3 or n % 2 == 0 or m not in NECKLACE_CONFIG or p % 2 == 0 or p > 0xFFFFFFFF
            or not 1 <= gap <= 0xFFFF or pow(omega, n, p) != 1 % p
            or any(n % q == 0 for q in range(3, int(n ** 0.5) + 1, 2))):
        raise ValueError("necklace preconditions not met (perm_modp_cuda.cu:955-968)")
    depth, threads, per_sm = NECKLACE_CONFIG[m]
    if m not in _frontiers:
        _frontiers[m] = necklace_frontier(m, depth)
    tasks_h = _frontiers[m]
    g = _smallest_primitive_root_prime(n)
    base, e = [], 1
    for _ in range(m):
        base.append(pow(omega, e, p))
        e = e * g % n
    base_sum = sum(base) % p
    tasks = torch.from_numpy(tasks_h.view(np.uint8)).cuda()
    dbase = torch.from_numpy(np.array(base, dtype=np.uint32).view(np.int32)).cuda()
    counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    raw = torch.zeros(1, dtype=torch.int64, device="cuda")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    d = driver()
    f = d.function("modp", k_necklace(m, depth))
    s = _stream(stream)
    if timer:
        timer.start(stream)
    d.launch(f, sms * per_sm, threads, threads * 4, s,
             [_ptr(tasks), ctypes.c_uint32(len(tasks_h)), _ptr(dbase), ctypes.c_uint32(base_sum),
              ctypes.c_uint32(p), ctypes.c_uint32(gap), _ptr(counter), _ptr(raw)])
    if timer:
        timer.stop(stream)
    r = (int(raw.cpu().item()) & ((1 << 64) - 1)) % p
    minor = r * pow((p >> 1) + 1, m, p) % p                   # :1092-1097
    return minor * (n % p) % p


def schur_gpu_primes(n: int):
    """perm_cuda.py:289-303, 372-404 (_plan_schur_crt_primes): descending odd
    primes q == 1 (mod n) below 2^32 until their product times the
    Graham-Lehmer modulus covers 2 * bound + 1."""
    sys.path.insert(0, str(HERE.parent / "rivin-perm_gb300"))
    from permgpu.crt import graham_lehmer_congruence, is_prime, schur_permanent_bound
    target = 2 * schur_permanent_bound(n) + 1
    cong = graham_lehmer_congruence(n)
    prod = cong[1] if cong else 1
    largest = (1 << 32) - 1
    c = largest - ((largest - 1) % n)
    if n % 2 == 1 and c % 2 == 0:
        c -= n
    step = n if n % 2 == 0 else 2 * n
    primes = []
    while prod < target and c >= 2:
        if is_prime(c):
            primes.append(c)
            prod *= c
        c -= step
    return primes, cong


# --- perm_binary_cuda.cu ---------------------------------------------------

B_MAX_ORDER = 63                                    # perm_binary_cuda.cu:31-35
B_VALUES = 2 * B_MAX_ORDER + 1
B_TARGET_TASKS = 1 << 20


def _orientation(m: np.ndarray, transpose: bool):
    """perm_binary_cuda.cu:256-297 (make_orientation): the densest column
    (first of the largest) keeps sign +1, the others go to Gray bits in
    increasing size (a stable order); the Gray cost weighs each column's size
    by how often its bit toggles."""
    n = m.shape[0]
    x = m.T if transpose else m
    columns = [[r for r in range(n) if x[r, c]] for c in range(n)]
    row_degrees = [int(x[r].sum()) for r in range(n)]
    fixed = 0
    for c in range(1, n):
        if len(columns[c]) > len(columns[fixed]):
            fixed = c
    variables = sorted((c for c in range(n) if c != fixed), key=lambda c: len(columns[c]))
    offsets, rows, cost = [0], [], 0
    for bit in range(n - 1):
        lst = columns[variables[bit]]
        rows.extend(lst)
        offsets.append(len(rows))
        cost += len(lst) << (n - 2 - bit)
    base = bytearray(64)
    for r in range(n):
        base[r] = row_degrees[r] & 0xFF
    return offsets, rows, bytes(base), cost


def _neg_inverse(p: int) -> int:                   # perm_binary_cuda.cu:226-234
    inv = p
    for _ in range(5):
        inv = (inv * (2 - p * inv)) & 0xFFFFFFFF
    return (-inv) & 0xFFFFFFFF


def _is_prime_u32(v: int) -> bool:
    if v < 2:
        return False
    if v % 2 == 0:
        return v == 2
    f = 3
    while f * f <= v:
        if v % f == 0:
            return False
        f += 2
    return True


def binary_modp(matrix, p: int, stream=None, timer=None) -> int:
    """perm_binary_cuda.cu:300-462 (binary_permanent_modp_cuda_impl): fixed-
    sign Glynn over 2^(n-1) states with packed signed-byte row sums, a zero
    counter and ratio-table Montgomery updates; odd prime n < p < 2^31."""
    import torch
    m = np.asarray(matrix)
    n = m.shape[0]
    if n < 0 or n > B_MAX_ORDER:
        raise ValueError(f"n must satisfy 0 <= n <= {B_MAX_ORDER}")
    if p <= n or p <= 2 or p >= (1 << 31) or not _is_prime_u32(p):
        raise ValueError("p must be an odd prime satisfying n < p < 2^31")
    if n == 0:
        return 1 % p
    if np.any((m != 0) & (m != 1)):
        raise ValueError("matrix entries must be 0 or 1")
    m = m.astype(np.uint8)
    if n == 1:
        return int(m[0, 0])
    if (m.sum(axis=1) == 0).any() or (m.sum(axis=0) == 0).any():
        return 0
    normal = _orientation(m, False)
    transposed = _orientation(m, True)
    offsets, rows, base, _ = transposed if transposed[3] < normal[3] else normal
    neg_inv = _neg_inverse(p)
    one_mont = (1 << 32) % p
    values = np.zeros(B_VALUES, np.uint32)
    trans = np.zeros((2, B_VALUES), np.uint32)
    for v in range(-B_MAX_ORDER, B_MAX_ORDER + 1):
        nv = v % p
        values[v + B_MAX_ORDER] = nv * one_mont % p
        for direction in (0, 1):
            nxt = v + (2 if direction else -2)
            if nxt < -B_MAX_ORDER or nxt > B_MAX_ORDER:
                continue
            nn = nxt % p
            if v == 0:
                ratio = nn
            else:
                inv = pow(nv, p - 2, p)
                ratio = inv if nxt == 0 else nn * inv % p
            trans[direction, v + B_MAX_ORDER] = ratio * one_mont % p
    d = driver()
    f, fname = d.function_containing("binary", "binary_glynn_ratio_kernel")
    # The constants live in the kernel's anonymous namespace; in device code
    # their names are also wrapped in the translation unit's internal
    # namespace: _ZN <_INTERNAL_H> <_GLOBAL__N__H> <name> E, H taken from
    # the kernel's name _ZN <len> _GLOBAL__N__H ...
    i = 3
    while fname[i].isdigit():
        i += 1
    ns = fname[i:i + int(fname[3:i])]
    h = ns[len("_GLOBAL__N__"):]
    internal = "_INTERNAL_" + h

    def cname(name):
        return [f"_ZN{len(internal)}{internal}{len(ns)}{ns}{len(name)}{name}E",
                f"_ZN{len(ns)}{ns}L{len(name)}{name}E", f"_ZN{len(ns)}{ns}{len(name)}{name}E"]
    off = np.zeros(B_MAX_ORDER, np.uint16)
    off[:len(offsets)] = offsets
    rw = np.zeros(B_MAX_ORDER * B_MAX_ORDER, np.uint8)
    rw[:len(rows)] = rows
    import torch
    torch.cuda.synchronize()                     # constants are shared by launches
    d.set_global("binary", cname("constant_offsets"), off.tobytes())
    d.set_global("binary", cname("constant_rows"), rw.tobytes())
    d.set_global("binary", cname("constant_base_words"), base)
    d.set_global("binary", cname("constant_value_mont"), values.tobytes())
    d.set_global("binary", cname("constant_transition"), trans.tobytes())
    states = 1 << (n - 1)
    task_count = min(states, B_TARGET_TASKS)
    per_task = states // task_count
    blocks = (task_count + 255) // 256
    acc = torch.zeros(1, dtype=torch.int64, device="cuda")
    s = _stream(stream)
    if timer:
        timer.start(stream)
    d.launch(f, blocks, 256, 0, s,
             [ctypes.c_int(n), ctypes.c_uint32(p), ctypes.c_uint32(neg_inv), ctypes.c_uint32(one_mont),
              ctypes.c_uint64(states), ctypes.c_uint64(per_task), ctypes.c_uint64(task_count),
              _ptr(acc)])
    if timer:
        timer.stop(stream)
    total = int(acc.cpu().item()) & ((1 << 64) - 1)
    summed = total % p
    # Montgomery form out (multiply by 1), then 2^(1-n): :443-451
    unscaled = summed * pow(1 << 32, -1, p) % p
    return unscaled * pow((p >> 1) + 1, n - 1, p) % p


# --- perm_parallel_cuda.cu -------------------------------------------------

def parallel_real(matrix, stream=None, timer=None) -> float:
    """perm_parallel_cuda.cu:343-414 (permanent_parallel_real): FP64 Glynn,
    Kahan-compensated per thread, then passes of reduce_kernel and 2^(1-n)."""
    import torch
    a = np.ascontiguousarray(matrix, dtype=np.float64)
    n = a.shape[0]
    if n <= 0 or n > 63:
        raise ValueError("n out of range [1,63]")
    if n == 1:
        return float(a[0, 0])
    total = 1 << (n - 1)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    total_threads = 1024 if n <= 20 else sms * 128 if n <= 30 else sms * 256
    blocks = (total_threads + 127) // 128
    total_threads = blocks * 128
    iters = (total + total_threads - 1) // total_threads
    mat = torch.from_numpy(a.ravel()).cuda()
    partial = torch.empty(total_threads, dtype=torch.float64, device="cuda")
    d = driver()
    s = _stream(stream)
    if timer:
        timer.start(stream)
    d.launch(d.function("parallel", K_F64), blocks, 128, 0, s,
             [_ptr(mat), ctypes.c_uint64(0), ctypes.c_int(n), ctypes.c_uint64(total),
              ctypes.c_uint64(iters), _ptr(partial), ctypes.c_uint64(0)])
    # reduce_host (perm_parallel_cuda.cu:254-338): 256-thread passes
    fr = d.function("parallel", K_F64_REDUCE)
    nb0 = (total_threads + 255) // 256
    s1 = torch.empty(nb0, dtype=torch.float64, device="cuda")
    s2 = torch.empty(nb0, dtype=torch.float64, device="cuda")
    src, dst, cur = partial, s1, total_threads
    while cur > 1:
        nb = (cur + 255) // 256
        d.launch(fr, nb, 256, 256 * 8, s,
                 [_ptr(src), ctypes.c_uint64(0), ctypes.c_uint64(cur), _ptr(dst), ctypes.c_uint64(0)])
        src = dst
        dst = s2 if dst is s1 else s1
        cur = nb
    if timer:
        timer.stop(stream)
    return math.ldexp(float(src[:1].cpu().item()), -(n - 1))


class Timer:
    """CUDA events around the reference's device work on the launch stream."""

    def __init__(self):
        self.ms = []

    def start(self, stream=None):
        import torch
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e0.record(stream or torch.cuda.current_stream())

    def stop(self, stream=None):
        import torch
        e1 = torch.cuda.Event(enable_timing=True)
        e1.record(stream or torch.cuda.current_stream())
        e1.synchronize()
        self.ms.append(self.e0.elapsed_time(e1))


def _reference_primes(bound: int):
    """perm.py:1116-1127: primes upward from 2^30 until their product
    exceeds 2 * bound + 1."""
    sys.path.insert(0, str(HERE.parent / "rivin-perm_gb300"))
    from permgpu.crt import is_prime
    primes, prod, c = [], 1, 1 << 30
    while prod < 2 * bound + 1:
        if is_prime(c):
            primes.append(c)
            prod *= c
        c += 1
    return primes


def _pm32_primes(bound: int):
    """Primes 2^32 - c (c < 2^16), descending, covering 2 * bound + 1."""
    sys.path.insert(0, str(HERE.parent / "rivin-perm_gb300"))
    from permgpu.crt import is_prime
    primes, prod, c = [], 1, 1
    while prod < 2 * bound + 1:
        if is_prime((1 << 32) - c):
            primes.append((1 << 32) - c)
            prod *= (1 << 32) - c
        c += 2
    return primes


def main(argv=None):
    """Times the reference's CUDA kernels on the benchmark workloads; one
    JSON line per measurement.  Results are checked against this
    repository's exact engine."""
    import argparse
    import json
    import time
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--workloads", default="generic24,generic32,batch4096,schur41,grid40,binary40,float28")
    ap.add_argument("--f64-sample", type=int, default=4)
    args = ap.parse_args(argv)
    root = HERE.parent
    sys.path.insert(0, str(root / "rivin-perm_gb300"))
    sys.path.insert(0, str(root))
    from permgpu import _lib, workloads
    from permgpu.crt import matrix_permanent_bound, signed_lift
    if not available():
        print(json.dumps({"unavailable": "reference cubins not built (oracle/build_ref.sh)"}))
        return
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    todo = args.workloads.split(",")

    def line(**kw):
        print(json.dumps(kw), flush=True)

    for wl in ("generic24", "generic32"):
        if wl not in todo:
            continue
        a = workloads.generic24() if wl == "generic24" else workloads.generic32()
        n = a.shape[0]
        want = _lib.exact_permanent(a, _lib.exact_limbs(a))
        bound = matrix_permanent_bound(a.tolist())
        for kind, primes, fn in (("ryser_modp (permanent_modp_cuda)", _reference_primes(bound), permanent_modp),
                                 ("glynn_pm32 (permanent_glynn_modp_pm32_kernel)", _pm32_primes(bound),
                                  glynn_modp)):
            if n not in PM32_ORDERS and "pm32" in kind:
                kind = "glynn_modp (permanent_glynn_modp_kernel)"
            t = Timer()
            t0 = time.perf_counter()
            res = [fn(a, p, stream, t) for p in primes]
            wall = time.perf_counter() - t0
            got = signed_lift(res, primes, bound)
            line(workload=wl, reference_kernel=kind, primes=len(primes), prime_bits=primes[0].bit_length(),
                 device_ms_per_prime=t.ms, device_s_total=sum(t.ms) / 1e3, wall_s=wall,
                 exact_result_matches=got == want)
    if "batch4096" in todo:
        # the reference's own per-matrix GPU loop (one call per matrix and CRT
        # prime, perm.py:1116-1127 primes) estimated from one matrix of each
        # order: per-order time x the batch's count of that order
        mats = workloads.batch4096()
        by_order = {}
        for m in mats:
            by_order.setdefault(m.shape[0], []).append(m)
        for kind, fn in (("ryser_modp (permanent_modp_cuda)", permanent_modp),
                         ("glynn_modp (permanent_glynn_modp_kernel)", glynn_modp)):
            est, ok, sample_s = 0.0, True, 0.0
            for n, group in sorted(by_order.items()):
                a = group[0]
                bound = matrix_permanent_bound(a.tolist())
                primes = _reference_primes(bound)
                t = Timer()
                res = [fn(a, q, stream, t) for q in primes]
                ok &= signed_lift(res, primes, bound) == _lib.exact_permanent(a, _lib.exact_limbs(a))
                dt = sum(t.ms) / 1e3
                sample_s += dt
                est += dt * len(group)
            line(workload="batch4096", reference_kernel=kind,
                 estimate="one matrix of each order 12..28 timed (all its primes), "
                          "times the batch's count of that order",
                 sample_device_s=sample_s, est_device_s_for_batch=est, exact_results_match=ok)
    if "schur41" in todo:
        from permgpu.crt import crt, nth_root_of_unity, schur_permanent_bound
        n = 41
        want = int(json.loads((root / "tests" / "golden" / "schur.json").read_text())["table"][str(n)])
        primes, cong = schur_gpu_primes(n)
        t = Timer()
        t0 = time.perf_counter()
        res, ok = [], True
        for q in primes:
            w = nth_root_of_unity(n, q)
            r = schur_necklace_modp(n, w, q, stream, t)
            ok &= r == _lib.schur_residues(n, [q], [w])[0]
            res.append(r)
        wall = time.perf_counter() - t0
        mods = primes + ([cong[1]] if cong else [])
        rs = res + ([cong[0]] if cong else [])
        x, mm = crt(rs, mods), 1
        for q in mods:
            mm *= q
        got = x - mm if x > schur_permanent_bound(n) else x
        line(workload="schur41", reference_kernel="schur_necklace_pm32_kernel<40,24> "
             "(schur_permanent_modp_cuda)", primes=len(primes), device_ms_per_prime=t.ms,
             device_s_total=sum(t.ms) / 1e3, wall_s=wall, residues_match=ok,
             exact_result_matches=got == want)
    bins = {}
    if "grid40" in todo:
        import json as _j
        g = _j.loads((root / "tests" / "golden" / "binary.json").read_text())
        bins["grid40"] = np.array(g["grid_4x4x5_periodic01"]["matrix"], dtype=np.int64)
    if "binary40" in todo:
        bins["binary40[0]"] = workloads.binary40(1)[0].astype(np.int64)
    for wl, m in bins.items():
        p = 2_147_483_647
        ours = _lib.binary_residues(m, [p])[0]
        t = Timer()
        t0 = time.perf_counter()
        r = binary_modp(m, p, stream, t)
        line(workload=wl, reference_kernel="binary_glynn_ratio_kernel (binary_permanent_modp_cuda)",
             prime=p, device_s=t.ms[0] / 1e3, wall_s=time.perf_counter() - t0,
             residue_matches=r == ours)
    if "float28" in todo:
        mats = workloads.float28(256)[: args.f64_sample]
        t = Timer()
        vals = [parallel_real(m, stream, t) for m in mats]
        ours, _, _ = _lib.glynn_f64_fwd_bwd(np.asarray(mats), want_grad=False)
        err = max(abs(v - float(o)) / max(1e-300, abs(float(o))) for v, o in zip(vals, np.ravel(ours)))
        line(workload="float28 forward", reference_kernel="permanent_glynn_kernel<false> (permanent_parallel_real)",
             matrices=len(mats), device_ms_per_matrix=t.ms, est_s_for_256=256 * sum(t.ms) / len(t.ms) / 1e3,
             max_rel_diff_vs_ours=err)


if __name__ == "__main__":
    main()
