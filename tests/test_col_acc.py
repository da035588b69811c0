"""CPU: the inline-PTX carry chains of col_acc.cuh (the exact kernel's
signed multi-word products MulWordS and column folds FoldCols).

Each asm block is executed by a small interpreter of the PTX it uses
(mul.wide.u32/s32, mov.b64 pack/unpack, add.cc/addc.cc/addc, shr.s32) on
random and extreme operands and compared with Python integers; the header
must also be exactly what gen_col_acc.py writes."""

import importlib.util
import random
import re
import shutil
from pathlib import Path

CSRC = Path(__file__).resolve().parents[1] / "rivin-perm_gb300" / "csrc"
M32 = (1 << 32) - 1
M64 = (1 << 64) - 1


def _blocks(src, kind):
    pat = re.compile(r"struct %s<([0-9, ]+)> \{.*?asm\(\"\{\\n\\t\"\n(.*?)\"\}\"\n\s*: (.*?)\n"
                     r"\s*: (.*?)\);" % kind, re.S)
    for m in pat.finditer(src):
        params = [int(x) for x in m.group(1).split(",")]
        lines = [l.strip().strip('"').replace("\\n\\t", "").strip()
                 for l in m.group(2).splitlines()]
        yield params, [l for l in lines if l]


def _s32(v):
    v &= M32
    return v - (1 << 32) if v >> 31 else v


def _run(lines, ops):
    regs, cc = {}, 0

    def val(x):
        x = x.strip()
        if x.startswith("%"):
            return ops[int(x[1:])]
        if re.fullmatch(r"-?\d+", x):
            return int(x)
        return regs[x]

    for line in lines:
        if line.startswith(".reg"):
            continue
        op, rest = line.split(None, 1)
        rest = rest.rstrip(";")
        if op == "mov.b64":
            m = re.match(r"\{(\w+), (\w+)\}, (%\d+|\w+)$", rest)
            v = val(m.group(3)) & M64
            regs[m.group(1)], regs[m.group(2)] = v & M32, v >> 32
            continue
        args = [a.strip() for a in rest.split(",")]
        a = [val(x) for x in args[1:]]
        if op == "mul.wide.u32":
            r = (a[0] & M32) * (a[1] & M32)
        elif op == "mul.wide.s32":
            r = (_s32(a[0]) * _s32(a[1])) & M64
        elif op == "mov.b32":
            r = a[0] & M32
        elif op == "shr.s32":
            r = (_s32(a[0]) >> a[1]) & M32
        elif op in ("add.cc.u32", "addc.cc.u32", "addc.u32"):
            t = (a[0] & M32) + (a[1] & M32) + (cc if op.startswith("addc") else 0)
            r = t & M32
            if ".cc" in op:
                cc = t >> 32
        else:
            raise ValueError(op)
        if args[0].startswith("%"):
            ops[int(args[0][1:])] = r
        else:
            regs[args[0]] = r
    return ops


def _signed(words):
    v = sum((w & M32) << (32 * i) for i, w in enumerate(words))
    return v - (1 << (32 * len(words))) if words[-1] >> 31 else v


def test_header_is_what_the_generator_writes(tmp_path):
    shutil.copy(CSRC / "gen_col_acc.py", tmp_path / "gen_col_acc.py")
    spec = importlib.util.spec_from_file_location("gen_col_acc", tmp_path / "gen_col_acc.py")
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    gen.main()
    assert (tmp_path / "col_acc.cuh").read_text() == (CSRC / "col_acc.cuh").read_text()


def test_signed_word_products_are_exact():
    # R (L words, top word signed, |R| < 2^(31 L)) times 0 <= y < 2^31
    src = (CSRC / "col_acc.cuh").read_text()
    rng = random.Random(1)
    blocks = list(_blocks(src, "MulWordS"))
    assert [b[0][0] for b in blocks] == list(range(1, 16))
    for (L,), lines in blocks:
        extremes = [0, 1, -1, (1 << (31 * L)) - 1, -(1 << (31 * L)) + 1]
        for trial in range(400):
            bits = rng.randint(1, 31 * L)
            r = rng.randint(-(1 << bits) + 1, (1 << bits) - 1) if trial >= 5 else extremes[trial]
            y = rng.choice([0, 1, (1 << 31) - 1, rng.randint(0, (1 << 31) - 1)])
            words = [(r >> (32 * i)) & M32 for i in range(L)]
            ops = _run(lines, words + [0, y])
            assert _signed(ops[:L + 1]) == r * y, (L, r, y)


def test_column_folds_add_exactly():
    # acc (NL words) += sum_l col[l] 2^(32 l) + colt 2^(32 (NR-1)), modulo 2^(32 NL)
    src = (CSRC / "col_acc.cuh").read_text()
    rng = random.Random(2)
    blocks = list(_blocks(src, "FoldCols"))
    assert len(blocks) == 42
    for (NR, NL), lines in blocks:
        W = 1 << (32 * NL)
        for _ in range(200):
            acc = rng.randint(-(1 << (32 * NL - 8)), 1 << (32 * NL - 8))
            cols = [rng.choice([0, M64, rng.randint(0, M64)]) for _ in range(NR - 1)]
            colt = rng.choice([-(1 << 63), (1 << 63) - 1, 0, -1,
                               rng.randint(-(1 << 63), (1 << 63) - 1)])
            ops = [(acc >> (32 * i)) & M32 for i in range(NL)] + cols + [colt & M64]
            got = _signed(_run(lines, ops)[:NL])
            want = acc + sum(c << (32 * i) for i, c in enumerate(cols)) + (colt << (32 * (NR - 1)))
            assert (got - want) % W == 0, (NR, NL)
