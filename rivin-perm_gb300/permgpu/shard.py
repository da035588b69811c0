"""Sharding one permanent across ranks / hosts.

The Glynn sum is a sum over 2^(n-1) independent Gray states, so any
partition of the state range into contiguous pieces gives partial sums that
simply add: per(A) = 2^(1-n) * sum_ranks S_rank.  There is no device
collective: each rank evaluates its range (pg_exact_partial on its GPU),
and the exchange is a host-level gather of a few 64-bit words per rank.

    lo, hi = state_range(n, rank, world)
    words = exact_partial_words(A, lo, hi)          # on the rank's GPU
    all = gather(words)                              # any transport
    per = combine_exact_words(all, n)

split_exact_permanent runs these steps on one rank with a torch.distributed
all-gather as the transport.  The same split works for residues
(combine_residues).
"""

from __future__ import annotations

import ctypes
from typing import Iterable, List, Sequence, Tuple

import numpy as np

from . import _lib


def state_range(n: int, rank: int, world: int, align: int = 64) -> Tuple[int, int]:
    """Contiguous, balanced slice [lo, hi) of the 2^(n-1) Gray states for
    `rank` of `world`, with boundaries on multiples of `align` (a power of
    two) so every slice is a whole number of aligned chunks."""
    states = 1 << max(n - 1, 0)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    align = min(align, states)
    units = states // align
    lo = rank * units // world * align
    hi = (rank + 1) * units // world * align
    return lo, hi


def exact_partial_words(matrix, lo: int, hi: int) -> List[int]:
    """Unscaled per-word sums of the Glynn terms over states [lo, hi) from
    the exact GPU engine (word w has weight 2^(32 w), last word signed)."""
    a = np.ascontiguousarray(matrix, dtype=np.int64)
    out = np.zeros(32, dtype=np.int64)
    nw = ctypes.c_int()
    _lib.check(_lib.load().pg_exact_partial(_lib.ptr(a, ctypes.c_int64), a.shape[0],
                                            ctypes.c_uint64(lo), ctypes.c_uint64(hi),
                                            _lib.ptr(out, ctypes.c_int64), 32,
                                            ctypes.byref(nw)))
    return [int(x) for x in out[: nw.value]]


def words_value(words: Sequence[int]) -> int:
    return sum(int(w) << (32 * i) for i, w in enumerate(words))


def combine_exact_words(word_lists: Iterable[Sequence[int]], n: int) -> int:
    """per(A) from the ranks' partial words (checks 2^(n-1) divides the sum)."""
    total = sum(words_value(w) for w in word_lists)
    if n >= 1 and total % (1 << (n - 1)):
        raise RuntimeError("partial sums do not add up to a multiple of 2^(n-1)")
    return total >> max(n - 1, 0)


def residue_partials(matrix, lo: int, hi: int, moduli: Sequence[int]) -> List[int]:
    """Unscaled Glynn sums over Gray states [lo, hi) modulo each odd modulus
    below 2^32 (pg_residues_partial); combine_residues turns the values of a
    partition of [0, 2^(n-1)) into per(A) mod p."""
    a = np.ascontiguousarray(matrix, dtype=np.int64)
    mods = np.ascontiguousarray([int(m) for m in moduli], dtype=np.uint64)
    out = np.zeros(len(mods), dtype=np.uint64)
    _lib.check(_lib.load().pg_residues_partial(_lib.ptr(a, ctypes.c_int64), a.shape[0],
                                               ctypes.c_uint64(lo), ctypes.c_uint64(hi),
                                               _lib.ptr(mods, ctypes.c_uint64), len(mods),
                                               _lib.ptr(out, ctypes.c_uint64)))
    return [int(x) for x in out]


def combine_residues(partials: Iterable[int], p: int, n: int) -> int:
    """per(A) mod odd p from unscaled partial Glynn sums mod p."""
    total = sum(int(x) for x in partials) % p
    inv2 = (p + 1) // 2
    return total * pow(inv2, n - 1, p) % p


GATHER_WIDTH = 32      # words per rank in the exchange (NL <= 18 for every shape)


def torch_gather(words: Sequence[int], group=None) -> List[List[int]]:
    """All-gather one rank's partial words over torch.distributed (host
    tensors for gloo, device tensors for nccl); returns every rank's words."""
    import torch
    import torch.distributed as dist
    if len(words) > GATHER_WIDTH:
        raise ValueError("too many partial words for the exchange")
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor(list(words) + [0] * (GATHER_WIDTH - len(words)), dtype=torch.int64,
                     device=dev)
    out = [torch.zeros_like(t) for _ in range(dist.get_world_size(group))]
    dist.all_gather(out, t, group=group)
    return [o.cpu().tolist() for o in out]


def split_exact_permanent(matrix, rank: int, world: int, gather=torch_gather,
                          partial=exact_partial_words) -> int:
    """per(A) of one matrix split across `world` ranks: this rank walks its
    Gray range on its GPU (`partial`), the words are exchanged (`gather`,
    any transport), and every rank combines the same exact value."""
    n = len(matrix)
    lo, hi = state_range(n, rank, world)
    words = partial(matrix, lo, hi)
    return combine_exact_words(gather(words), n)
