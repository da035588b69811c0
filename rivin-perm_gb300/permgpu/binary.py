"""Binary (0/1) perfect-matching counts on the GPU.

Host preprocessing keeps the contract of rivin-perm perm_binary.py:
strict 0/1 validation (:173-215), a perfect matching by augmenting paths
(:609-655), strongly connected components of the matching digraph
(:658-706) splitting the matrix into independent square blocks
(:709-752), and per-block exact evaluation.  Each block goes to the exact
GPU engine when its row-sum bound fits, else to GPU residues modulo
descending 31-bit primes with the incremental Garner lift of
perm_binary.py:843-863 (which raises if the lift leaves [0, bound]).
"""

from __future__ import annotations

import math
import operator
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .crt import binary_block_bound, binary_primes_above, is_prime


def normalize_binary_matrix(matrix, *, strict: bool = True) -> Tuple[Tuple[int, ...], ...]:
    if not isinstance(strict, bool):
        raise TypeError("strict must be a boolean")
    shape = getattr(matrix, "shape", None)
    if shape is not None:
        shape = tuple(shape)
        if len(shape) != 2:
            raise ValueError("matrix must be two-dimensional")
        if shape[0] != shape[1]:
            raise ValueError("matrix must be square")
    try:
        n = len(matrix)
    except TypeError as exc:
        raise TypeError("matrix must be a sequence of rows") from exc
    rows = []
    for i, row in enumerate(matrix):
        try:
            width = len(row)
        except TypeError as exc:
            raise TypeError("matrix rows must be sequences") from exc
        if width != n:
            raise ValueError("matrix must be square")
        out = []
        for j, entry in enumerate(row):
            if isinstance(entry, (bool, np.bool_)):
                v = int(entry)
            else:
                try:
                    v = int(operator.index(entry))
                except TypeError as exc:
                    raise TypeError(
                        "binary matrix entries must be integers; "
                        f"entry ({i}, {j}) is {type(entry).__name__}") from exc
            if strict and v not in (0, 1):
                raise ValueError(
                    "binary matrix entries must be 0 or 1 in strict mode; "
                    f"entry ({i}, {j}) is {v}")
            out.append(1 if v else 0)
        rows.append(tuple(out))
    if len(rows) != n:
        raise ValueError("matrix row count changed during validation")
    return tuple(rows)


def row_masks(matrix) -> List[int]:
    return [sum(1 << j for j, v in enumerate(row) if v) for row in matrix]


def perfect_matching(masks: Sequence[int]) -> Optional[List[int]]:
    """Row -> column perfect matching by BFS augmenting paths, or None."""
    n = len(masks)
    match_row, match_col = [-1] * n, [-1] * n
    for root in range(n):
        parent = [-1] * n            # column -> row that reached it
        seen_col = [False] * n
        queue, head, free = [root], 0, -1
        visited_row = [False] * n
        visited_row[root] = True
        while head < len(queue) and free < 0:
            r = queue[head]
            head += 1
            m = masks[r]
            while m:
                low = m & -m
                c = low.bit_length() - 1
                m ^= low
                if seen_col[c]:
                    continue
                seen_col[c] = True
                parent[c] = r
                if match_col[c] < 0:
                    free = c
                    break
                nr = match_col[c]
                if not visited_row[nr]:
                    visited_row[nr] = True
                    queue.append(nr)
        if free < 0:
            return None
        c = free
        while c >= 0:
            r = parent[c]
            prev = match_row[r]
            match_row[r], match_col[c] = c, r
            c = prev
    return match_row


def strong_components(adj: Sequence[Sequence[int]]) -> List[List[int]]:
    """Iterative Tarjan SCC; components returned with sorted members."""
    n = len(adj)
    index = [0] * n
    low = [0] * n
    on = [False] * n
    seen = [False] * n
    stack: List[int] = []
    comps: List[List[int]] = []
    counter = 0
    for s in range(n):
        if seen[s]:
            continue
        work = [(s, 0)]
        seen[s] = True
        index[s] = low[s] = counter
        counter += 1
        stack.append(s)
        on[s] = True
        while work:
            v, i = work[-1]
            if i < len(adj[v]):
                work[-1] = (v, i + 1)
                w = adj[v][i]
                if not seen[w]:
                    seen[w] = True
                    index[w] = low[w] = counter
                    counter += 1
                    stack.append(w)
                    on[w] = True
                    work.append((w, 0))
                elif on[w]:
                    low[v] = min(low[v], index[w])
            else:
                work.pop()
                if work:
                    u = work[-1][0]
                    low[u] = min(low[u], low[v])
                if low[v] == index[v]:
                    comp = []
                    while True:
                        w = stack.pop()
                        on[w] = False
                        comp.append(w)
                        if w == v:
                            break
                    comps.append(sorted(comp))
    return comps


def matching_blocks(masks: Sequence[int]) -> Tuple[bool, List[List[List[int]]]]:
    """(feasible, blocks): independent square 0/1 blocks whose permanents
    multiply to per(A); an infeasible matrix (no perfect matching) has
    permanent 0."""
    n = len(masks)
    match = perfect_matching(masks)
    if match is None:
        return False, []
    if n == 0:
        return True, []
    col_to_row = [-1] * n
    for r, c in enumerate(match):
        col_to_row[c] = r
    adj = []
    for m in masks:
        targets = []
        while m:
            low = m & -m
            targets.append(col_to_row[low.bit_length() - 1])
            m ^= low
        adj.append(targets)
    blocks = []
    for comp in strong_components(adj):
        cols = [match[r] for r in comp]
        blocks.append([[(masks[r] >> c) & 1 for c in cols] for r in comp])
    return True, blocks


def _validate_prime(p, order: int) -> int:
    if isinstance(p, bool) or not isinstance(p, int):
        try:
            p = operator.index(p)
        except TypeError as exc:
            raise TypeError("p must be an integer") from exc
    p = int(p)
    if p <= 1:
        raise ValueError("p must be greater than 1")
    if p == 2 or p <= order or not is_prime(p):
        raise ValueError("modulus must be an odd prime greater than the matrix order")
    return p


def _block_exact(block: List[List[int]]) -> int:
    n = len(block)
    if n == 1:
        return block[0][0]
    bound = binary_block_bound(block)
    arr = np.asarray(block, dtype=np.int64)
    if _lib.exact_supported(arr):
        return _lib.exact_permanent(arr, _lib.exact_limbs(arr))
    primes = binary_primes_above(bound)
    res = _lib.binary_residues(np.asarray(block, dtype=np.uint8), primes)
    value, product = 0, 1
    for p, r in zip(primes, res):
        value += product * ((r - value) % p * pow(product, -1, p) % p)
        product *= p
    if value > bound:
        raise RuntimeError("binary residues reconstructed outside the bound")
    return value


def binary_permanent(matrix, *, backend: str = "auto", parallel: bool = True,
                     num_threads: int = 0, strict: bool = True) -> int:
    """Exact permanent of a square 0/1 matrix (perm_binary.py:943-1005 API)."""
    if not isinstance(parallel, bool):
        raise TypeError("parallel must be a boolean")
    if not isinstance(backend, str):
        raise TypeError("backend must be a string")
    if backend.lower() not in ("auto", "native", "gpu"):
        raise ValueError("backend must be one of: 'auto', 'native', 'gpu'")
    rows = normalize_binary_matrix(matrix, strict=strict)
    if not rows:
        return 1
    if len(rows) == 1:
        return rows[0][0]
    feasible, blocks = matching_blocks(row_masks(rows))
    if not feasible:
        return 0
    result = 1
    for block in blocks:
        result *= _block_exact(block)
    return result


def binary_permanent_mod_p(matrix, p: int, *, backend: str = "auto",
                           parallel: bool = True, num_threads: int = 0,
                           strict: bool = True) -> int:
    """per(A) mod an odd prime p > n (perm_binary.py:893-940 API)."""
    rows = normalize_binary_matrix(matrix, strict=strict)
    p = _validate_prime(p, len(rows))
    if not rows:
        return 1 % p
    if len(rows) == 1:
        return rows[0][0] % p
    feasible, blocks = matching_blocks(row_masks(rows))
    if not feasible:
        return 0
    result = 1
    for block in blocks:
        if len(block) == 1:
            continue
        r = _lib.binary_residues(np.asarray(block, dtype=np.uint8), [p])[0]
        result = result * r % p
    return result


def binary_permanent_bound(matrix, *, strict: bool = True) -> int:
    rows = normalize_binary_matrix(matrix, strict=strict)
    feasible, blocks = matching_blocks(row_masks(rows))
    if not feasible:
        return 0
    return math.prod(binary_block_bound(b) for b in blocks) if blocks else 1
