"""Exact planning around the residue engines: bounds, prime plans, CRT.

Pure Python integer arithmetic (arbitrary precision); the exponential work
happens on the GPU.  Each function names the rivin-perm routine whose
contract it keeps.
"""

from __future__ import annotations

import math
from typing import List, Optional, Sequence, Tuple

# Witness set deterministic for all 64-bit integers (the set rivin-perm uses
# in perm.py:162-195).
_MR_WITNESSES = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)

# Odd moduli below this run the 32-bit Montgomery kernel.
FAST_PRIME_LIMIT = 1 << 31
# The necklace kernel (Schur permanents of prime order) sums row sums lazily
# and needs moduli below 2^30; it takes over from order 37 on.
NECKLACE_PRIME_LIMIT = 1 << 30
NECKLACE_AUTO_MIN_ORDER = 37


def is_prime(n: int) -> bool:
    """Deterministic Miller-Rabin for n < 3.3e24 (perm.py:162-195 contract)."""
    if n < 2:
        return False
    for p in _MR_WITNESSES:
        if n == p:
            return True
        if n % p == 0:
            return False
    d, r = n - 1, 0
    while d % 2 == 0:
        d //= 2
        r += 1
    for a in _MR_WITNESSES:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(r - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def matrix_permanent_bound(matrix: Sequence[Sequence[int]]) -> int:
    """prod_i max(1, sum_j |a_ij|) — the bound of perm.py:939-953."""
    bound = 1
    for row in matrix:
        bound *= max(1, sum(abs(int(x)) for x in row))
    return bound


def descending_primes(target: int, limit: int = FAST_PRIME_LIMIT,
                      congruent_mod: int = 1) -> List[int]:
    """Largest primes p < limit with p == 1 (mod congruent_mod) until their
    product reaches ``target``.  Any prime set whose product covers the
    signed range reconstructs the same integer (the CRT lift is unique), so
    the plan is free to use the widest primes the fast kernel accepts."""
    primes: List[int] = []
    product = 1
    step = congruent_mod
    c = limit - 1
    c -= (c - 1) % step            # c == 1 (mod step)
    if step % 2 == 1 and c % 2 == 0:
        c -= step                  # keep odd candidates only
    if step % 2 == 1:
        step *= 2
    while product < target:
        if c < 3:
            raise ValueError("ran out of CRT primes below the limit")
        if is_prime(c):
            primes.append(c)
            product *= c
        c -= step
    return primes


def crt(residues: Sequence[int], moduli: Sequence[int]) -> int:
    """Garner lift into [0, prod(moduli)) — perm.py:542-584 contract."""
    if len(residues) != len(moduli):
        raise ValueError("residues and moduli must have the same length")
    if not residues:
        return 0
    result, mod = int(residues[0]) % int(moduli[0]), int(moduli[0])
    for r, m in zip(residues[1:], moduli[1:]):
        m = int(m)
        if math.gcd(mod, m) != 1:
            raise ValueError("Moduli must be pairwise coprime")
        t = (int(r) - result) * pow(mod, -1, m) % m
        result += mod * t
        mod *= m
    return result


def signed_lift(residues: Sequence[int], moduli: Sequence[int], bound: int) -> int:
    """CRT then the sign rule of perm.py:1207-1210 (result > bound => negative)."""
    value = crt(residues, moduli)
    product = math.prod(int(m) for m in moduli)
    if value > bound:
        value -= product
    return value


# ---- Schur planning (perm.py:262-326, 587-605, 787-803) --------------------

def schur_permanent_bound(n: int) -> int:
    """ceil(n^(n/2)) in integer arithmetic (perm.py:587-605)."""
    if n == 0:
        return 1
    power = n ** n
    root = math.isqrt(power)
    return root if root * root == power else root + 1


def graham_lehmer_congruence(n: int) -> Optional[Tuple[int, int]]:
    """Theorem-only CRT congruence for odd Schur orders (perm.py:280-326):
    perm(S_n) == n! (mod n^3) for prime n >= 5; otherwise the product of the
    prime-power divisors p^((p^a-1) n / ((p-1) p^a)) with residue 0."""
    if n < 3 or not (n & 1):
        return None
    if n >= 5 and is_prime(n):
        modulus = n ** 3
        return math.factorial(n) % modulus, modulus
    remaining, modulus, p = n, 1, 3
    while p * p <= remaining:
        if remaining % p == 0:
            pa = 1
            while remaining % p == 0:
                remaining //= p
                pa *= p
            modulus *= p ** ((n // pa) * ((pa - 1) // (p - 1)))
        p += 2
    if remaining > 1:
        modulus *= remaining ** (n // remaining)
    return 0, modulus


def primitive_root(p: int) -> int:
    phi = p - 1
    factors, t, d = [], phi, 2
    while d * d <= t:
        if t % d == 0:
            factors.append(d)
            while t % d == 0:
                t //= d
        d += 1
    if t > 1:
        factors.append(t)
    for g in range(2, p):
        if all(pow(g, phi // q, p) != 1 for q in factors):
            return g
    raise ValueError(f"no primitive root for {p}")


def nth_root_of_unity(n: int, p: int) -> int:
    """A primitive n-th root of unity mod prime p == 1 (mod n) (perm.py:262-277)."""
    if (p - 1) % n:
        raise ValueError(f"p={p} is not == 1 (mod {n})")
    return pow(primitive_root(p), (p - 1) // n, p)


def uses_necklace(n: int) -> bool:
    """True when the automatic Schur dispatch evaluates perm(S_n) with the
    necklace quotient: n an odd prime with NECKLACE_AUTO_MIN_ORDER <= n < 64."""
    return NECKLACE_AUTO_MIN_ORDER <= n < 64 and is_prime(n)


def plan_schur(n: int, prime_limit: Optional[int] = None
               ) -> Tuple[List[int], Optional[Tuple[int, int]], int]:
    """GPU Schur plan: primes p == 1 (mod n) below `prime_limit` (2^30 for
    necklace orders, else 2^31), plus the Graham-Lehmer congruence used only
    at CRT time.  Returns (primes, congruence, bound)."""
    if prime_limit is None:
        prime_limit = NECKLACE_PRIME_LIMIT if uses_necklace(n) else FAST_PRIME_LIMIT
    bound = schur_permanent_bound(n)
    target = 2 * bound + 1
    congruence = graham_lehmer_congruence(n)
    if congruence is not None:
        target = -(-target // congruence[1])
    primes = descending_primes(target, prime_limit, n) if target > 1 else []
    return primes, congruence, bound


# ---- binary planning (perm_binary.py:538-606, 796-814) ---------------------

def ceil_nth_root(value: int, degree: int) -> int:
    if value <= 1 or degree == 1:
        return value
    lo, hi = 0, 1 << ((value.bit_length() + degree - 1) // degree)
    while lo + 1 < hi:
        mid = (lo + hi) // 2
        if pow(mid, degree) < value:
            lo = mid
        else:
            hi = mid
    return hi


def grouped_bregman_minc_bound(degrees: Sequence[int]) -> int:
    counts: dict = {}
    for d in degrees:
        if d == 0:
            return 0
        counts[d] = counts.get(d, 0) + 1
    bound = 1
    for d, c in counts.items():
        f = math.factorial(d)
        q, r = divmod(c, d)
        bound *= pow(f, q)
        if r:
            bound *= ceil_nth_root(pow(f, r), d)
    return bound


def binary_block_bound(block: Sequence[Sequence[int]]) -> int:
    """min(n!, row/column degree products, Bregman-Minc) (perm_binary.py:538-561)."""
    n = len(block)
    if n == 0:
        return 1
    rows = [sum(r) for r in block]
    cols = [sum(block[i][j] for i in range(n)) for j in range(n)]
    return min(math.factorial(n), math.prod(rows), math.prod(cols),
               grouped_bregman_minc_bound(rows), grouped_bregman_minc_bound(cols))


def binary_primes_above(bound: int) -> List[int]:
    """Descending primes from 2^31-1 with product > bound (perm_binary.py:796-814)."""
    primes, product, c = [], 1, (1 << 31) - 1
    while product <= bound:
        if is_prime(c):
            primes.append(c)
            product *= c
        c -= 2
    return primes
