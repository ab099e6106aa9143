"""The translator's bytecode, read back from the device, only ever holds
instructions of the opcode set of the kernel that will run it, and operands
inside the program's tile or dataset.  The evaluator's dispatch has no case
for anything else (it records a status bit and stops the walk); this checks
the invariant that case relies on, for every fixture and strategy, without
ever giving a kernel a bad instruction.

The instruction numbering restates the M_* enum of csrc/ppi_internal.cuh;
test_instruction_numbering_matches_the_header (CPU) keeps the two in step."""
import os
import re

import numpy as np
import pytest

from helpers import golden_names, load_golden, make_evaluator
from ppi_gpu import grammar as G

NAMES = golden_names()
HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "ppi-auto_gb300", "csrc",
                      "ppi_internal.cuh")

M = dict(M_END=0, M_LD_ROW=1, M_LD_C=2, M_PUSH=3, M_UN=4)
M["M_BR_L"] = M["M_UN"] + 25
M["M_BR_R"] = M["M_BR_L"] + 18
M["M_BC_L"] = M["M_BR_R"] + 18
M["M_BC_R"] = M["M_BC_L"] + 18
M["M_ITE"] = M["M_BC_R"] + 18
M["M_PUSH_LD"] = M["M_ITE"] + 6
M["M_COUNT"] = M["M_PUSH_LD"] + 1
DIRECT = 0x80000000
GENERIC_END = 0xFFFF
KIND_FAST, KIND_GENERIC, KIND_WIDE = 1, 2, 4

ARITH_UNARY = ["ABS", "POW2", "NEG", "EXP", "SIN", "COS", "SQRT", "LOG"]
ARITH_BINARY = ["ADD", "SUB", "MULT", "DIV"]
UNARY_FIRST, BINARY_FIRST = G.OP["NOT"], G.OP["AND"]


def allowed_ids(opset):
    """Instruction ids the kernel of an opcode set has a case for."""
    ids = {M["M_END"], M["M_LD_ROW"], M["M_LD_C"], M["M_PUSH"], M["M_PUSH_LD"]}
    un = [G.OP[n] for n in ARITH_UNARY] if opset == 1 else [o for o in range(UNARY_FIRST, len(G.OPS))]
    bi = [G.OP[n] for n in ARITH_BINARY] if opset == 1 else list(range(BINARY_FIRST, UNARY_FIRST))
    ids |= {M["M_UN"] + o - UNARY_FIRST for o in un}
    for fam in ("M_BR_L", "M_BR_R", "M_BC_L", "M_BC_R"):
        ids |= {M[fam] + o - BINARY_FIRST for o in bi}
    if opset == 0:
        ids |= {M["M_ITE"] + p for p in range(6)}
    return ids


def check_program(code, meta, opset, ncol, max_size):
    """Walk one program's code the way the kernel does; return a problem or None."""
    kind, rows, length = meta[0] & 0xFF, meta[0] >> 8, meta[1]
    if kind not in (KIND_FAST, KIND_WIDE, KIND_GENERIC):
        return None if length == 0 else "code for a program that does not run"
    if not 0 < length <= code.shape[0]:
        return "code length %d outside [1, %d]" % (length, code.shape[0])
    if kind == KIND_GENERIC:
        toks = code[1:length]
        if toks[-1, 0] != GENERIC_END:
            return "generic code does not end with its end marker"
        if (toks[:-1, 0] >= len(G.OPS)).any():
            return "generic token outside the op table"
        return None
    k, s, d = int(code[0, 0]), int(code[0, 1] & 0xFFFF), int(code[0, 1] >> 16)
    if k + s + 1 > rows:
        return "header needs %d rows, meta gives %d" % (k + s + 1, rows)
    cols = code[1:1 + (k + d + 1) // 2].reshape(-1)[:k + d]
    if len(cols) and (cols >= ncol).any():
        return "listed column outside the dataset's features"
    ok = allowed_ids(opset)
    pc = 1 + (k + d + 1) // 2
    row_ops = set(range(M["M_BR_L"], M["M_BC_L"])) | {M["M_LD_ROW"]}
    while pc < length:
        ins, imm = int(code[pc, 0]), int(code[pc, 1])
        if ins not in ok:
            return "instruction %d at %d outside opcode set %d" % (ins, pc, opset)
        if ins == M["M_END"]:
            return None if pc == length - 1 else "M_END before the end of the code"
        if ins in row_ops:
            if imm & DIRECT:
                if kind != KIND_WIDE or (imm & ~DIRECT) >= ncol:
                    return "direct column operand %x at %d" % (imm, pc)
            elif imm >= rows:
                return "row operand %d at %d beyond %d rows" % (imm, pc, rows)
        elif ins == M["M_PUSH"]:
            if imm >= s:
                return "push to row %d at %d, slots %d" % (imm, pc, s)
        elif ins == M["M_PUSH_LD"]:
            if (imm & 0xFFFF) >= s or (imm >> 16) >= rows:
                return "push/load rows %x at %d" % (imm, pc)
        elif M["M_ITE"] <= ins < M["M_PUSH_LD"]:
            if (imm & 0xFFFF) >= rows or (imm >> 16) >= rows:
                return "if-then-else rows %x at %d" % (imm, pc)
        pc += 1
    return "no M_END within the code length"


def test_instruction_numbering_matches_the_header():
    text = open(HEADER).read()
    body = re.search(r"enum : uint32_t \{(.*?)\};", text, re.S).group(1)
    env = {}
    for name, expr in re.findall(r"^\s*(M_\w+)\s*=\s*([^,/\n]+)", body, re.M):
        env[name] = eval(expr, {}, dict(env))
    assert env == M
    assert re.search(r"kDirectColumn = 0x80000000u", text)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("strat,lanes,math", [("PDP", 0, "fast"), ("PP", 0, "parity"),
                                               ("DP", 5, "native")])
def test_translator_output_stays_in_the_kernels_opcode_set(gpu_lib, name, strat, lanes, math):
    d = load_golden(name)
    for population in (len(d["size"]), 20000):   # one wave (widest tile) and occupancy tiles
        ev = make_evaluator(d, strat, lanes, math, population=population)
        ev.evaluate(d["phenotype"], d["ephemeral"], d["size"], 0.0)
        code, meta, opset = ev.translation(len(d["size"]))
        ncol = d["rows"].shape[1]
        for i in range(len(d["size"])):
            why = check_program(code[i], meta[i], opset, ncol, d["max_size"])
            assert why is None, (name, strat, population, i, why)
        ev.close()


@pytest.mark.gpu
def test_wide_programs_translate_within_the_opcode_set(gpu_lib):
    """Programs over 90 columns with a small main tile: wide-pass code with
    direct column operands."""
    from helpers import ProgramGen
    d = load_golden("allops")
    rng = np.random.default_rng(11)
    rows = rng.normal(0, 1, (600, 91)).astype(np.float32)
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.random(int(k)) for k in rng.integers(5, 80, 120)]
    ph, ep, sz = ProgramGen.rows(progs, 256)
    ev = make_evaluator(d, "PDP", 0, "fast", population=20000, max_size=256, rows=rows)
    ev.evaluate(ph, ep, sz, 0.0)
    code, meta, opset = ev.translation(len(sz))
    kinds = meta[:, 0] & 0xFF
    assert (kinds == KIND_WIDE).any()
    for i in range(len(sz)):
        why = check_program(code[i], meta[i], opset, rows.shape[1], 256)
        assert why is None, (i, why)
