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


def _bits(mask: int):
    while mask:
        low = mask & -mask
        yield low.bit_length() - 1
        mask ^= low


def perfect_matching(masks: Sequence[int]) -> Optional[List[int]]:
    """Row -> column perfect matching of the 0/1 matrix with row bitmasks
    `masks`, or None when there is none.

    Hopcroft-Karp in phases: a breadth-first pass from all unmatched rows at
    once assigns every row its alternating-path layer (row -> any column of
    the row -> the row matched to that column); a depth-first pass then
    augments a maximal set of vertex-disjoint paths that climb the layers
    and end at an unmatched column.  Each phase lengthens the shortest
    augmenting path, so O(sqrt(n)) phases suffice.
    """
    n = len(masks)
    col_of = [-1] * n            # row -> matched column
    row_of = [-1] * n            # column -> matched row
    while True:
        free_rows = [r for r in range(n) if col_of[r] < 0]
        if not free_rows:
            return col_of
        layer = [-1] * n
        for r in free_rows:
            layer[r] = 0
        frontier, open_cols, reached = free_rows, (1 << n) - 1, False
        while frontier and not reached:
            nxt = []
            for r in frontier:
                hit = masks[r] & open_cols
                open_cols &= ~hit
                for c in _bits(hit):
                    m = row_of[c]
                    if m < 0:
                        reached = True
                    elif layer[m] < 0:
                        layer[m] = layer[r] + 1
                        nxt.append(m)
            frontier = nxt
        if not reached:
            return None          # some row can reach no unmatched column
        todo = list(masks)       # columns each row has not tried yet
        grew = False
        for root in free_rows:
            rows, cols = [root], []
            while rows:
                r = rows[-1]
                step = None
                while todo[r]:
                    low = todo[r] & -todo[r]
                    todo[r] ^= low
                    c = low.bit_length() - 1
                    m = row_of[c]
                    if m < 0 or layer[m] == layer[r] + 1:
                        step = (c, m)
                        break
                if step is None:             # dead end: never revisit r
                    layer[r] = -1
                    rows.pop()
                    if cols:
                        cols.pop()
                    continue
                c, m = step
                cols.append(c)
                if m >= 0:
                    rows.append(m)
                    continue
                for rr, cc in zip(rows, cols):   # flip the path
                    col_of[rr], row_of[cc] = cc, rr
                for rr in rows:                  # vertex-disjoint paths per phase
                    layer[rr] = -1
                grew = True
                break
        if not grew:
            raise RuntimeError("matching phase found a free column but no augmenting path")


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
    permanent 0.

    The blocks are the fine decomposition of the bipartite graph: with a
    perfect matching fixed, orient every unmatched edge row -> column and
    every matched edge both ways; an edge lies on some perfect matching
    exactly when its ends share a strongly connected component, so the
    components (rows with their matched columns) are the blocks and every
    edge between components is in no perfect matching.  The decomposition
    does not depend on which perfect matching was found.
    """
    n = len(masks)
    match = perfect_matching(masks)
    if match is None:
        return False, []
    if n == 0:
        return True, []
    adj: List[List[int]] = [[] for _ in range(2 * n)]   # rows 0..n-1, columns n..2n-1
    for r, mask in enumerate(masks):
        adj[n + match[r]].append(r)
        adj[r].extend(n + c for c in _bits(mask))
    blocks = []
    for comp in strong_components(adj):
        rows = [v for v in comp if v < n]
        cols = sorted(match[r] for r in rows)
        blocks.append([[(masks[r] >> c) & 1 for c in cols] for r in rows])
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
