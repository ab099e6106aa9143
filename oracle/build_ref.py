#!/usr/bin/env python3
"""Build the reference's own hot-path code into oracle/_ref/ (test oracle only).

For each configuration below this recipe does what the reference's CMake build
does for one ``cmake -DGRAMMAR=... -DEF=... [-DCOST] [-DREDUCEMAX] [-DPROTECTED]
[-DNATIVE]`` (CMakeLists.txt:7-81), without running CMake:

1. runs the reference's script/read_grammar.py on the grammar, which writes the
   generated ``symbol``, ``grammar`` and ``interpreter_core`` headers;
2. configures src/definitions.h and src/costmatrix the way ``configure_file``
   does (``@EF@``, ``@COST@``, ``#cmakedefine``) and copies
   src/interpreter/functions.h beside them (src/interpreter/CMakeLists.txt:39-41);
3. compiles, from the sources where they lie under the reference tree:
   - libref_seq.so: src/interpreter/sequential.cc + oracle/ref_seq_driver.cc
   - libref_cl.so: src/interpreter/accelerator.cl as C++ through
     oracle/cl_shim.h + oracle/ref_cl_driver.cc
   - libref_decode.so: decode_rule/decode_real/decode cut out of src/ppi.cc
     (src/ppi.cc:106-182) + oracle/ref_decode_driver.cc.

Nothing here is part of the product; outputs go to oracle/_ref/ only (git
ignored).  The COST configurations pass a guarded error function through the
reference's own -DEF mechanism, because ``COST[(int)X][(int)Y]`` indexes out of
bounds whenever a prediction is not a class index: NaN X gives a NaN error and
each index is (int)v clamped to [0, N).

Usage: python3 oracle/build_ref.py [--ref TREE] [--only NAME ...]
The tree is --ref, else $PPI_REFERENCE, else the reference checkout this
recipe was written against (REFERENCE_DEFAULT).
"""
import argparse
import json
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
GRAMMARS = os.path.join(REPO, "ppi-auto_gb300", "grammars")
REFERENCE_DEFAULT = "/root/reference"


def reference_root():
    """The reference tree this recipe and the tests that read reference
    sources use: $PPI_REFERENCE when set, else REFERENCE_DEFAULT."""
    return os.environ.get("PPI_REFERENCE", REFERENCE_DEFAULT)

COST8 = ("[8]={{0,1.5,0.75,1.25,2,0.5,1,1.75},{1,0,1.5,0.5,0.75,2,1.25,0.6},"
         "{0.8,1.1,0,1.9,0.55,1.3,0.7,1.6},{1.4,0.65,1.2,0,1.05,0.9,1.8,0.5},"
         "{0.5,1.7,0.95,1.15,0,1.45,0.85,1.35},{1.25,0.7,1.6,0.8,1.9,0,0.6,1.1},"
         "{1.95,1.3,0.5,1.5,0.9,1.2,0,0.75},{0.6,0.85,1.75,1.05,1.4,0.55,1.65,0}}")
GUARDED_COST_EF = "ppi_guarded_cost_(COST, X, Y)"

# name: (grammar, EF, COST, REDUCEMAX, PROTECTED, NATIVE, MAX_PHENOTYPE_SIZE)
CONFIGS = {
    "iris": ("@ref/problem/iris/grammar.bnf", "((X)!=(Y))", None, 0, 1, 0, 64),
    "polynomial": ("@ref/problem/polynomial/grammar.bnf", "fabs((X)-(Y))", None, 0, 0, 0, 64),
    "random": ("@ref/problem/random/grammar.bnf", "fabs((X)-(Y))", None, 0, 1, 0, 128),
    "random_raw": ("@ref/problem/random/grammar.bnf", "fabs((X)-(Y))", None, 0, 0, 0, 128),
    "cfg1": ("config1_iris.bnf", "((X)!=(Y))", None, 0, 1, 0, 64),
    "cfg2": ("config2_poly.bnf", "fabs((X)-(Y))", None, 0, 1, 0, 128),
    "cfg2max": ("config2_poly.bnf", "fabs((X)-(Y))", None, 1, 1, 0, 128),
    "cfg4": ("config4_adjoint.bnf", "(((X)-(Y))*((X)-(Y)))", None, 0, 1, 0, 128),
    "cfg5": ("config5_stream.bnf", GUARDED_COST_EF, COST8, 0, 1, 0, 256),
    "allops": ("allops.bnf", "fabs((X)-(Y))", None, 0, 0, 0, 64),
    "allops_prot": ("allops.bnf", "fabs((X)-(Y))", None, 0, 1, 0, 64),
    "allops_sqmax": ("allops.bnf", "(((X)-(Y))*((X)-(Y)))", None, 1, 1, 0, 64),
}

GUARD_HELPER = """
/* ppi-oracle: guarded cost lookup used as -DEF for the COST configurations. */
template <int R, int C>
static inline float ppi_guarded_cost_(const float (&cost)[R][C], float x, float y) {
   if (x != x) return x;
   int ix = x >= (float)R ? R - 1 : (x > 0.0f ? (int)x : 0);
   int iy = y != y ? 0 : (y >= (float)C ? C - 1 : (y > 0.0f ? (int)y : 0));
   return cost[ix][iy];
}
"""


def grammar_path(ref, g):
    return g.replace("@ref", ref) if g.startswith("@ref") else os.path.join(GRAMMARS, g)


def configure(template, ef, cost, reducemax, protected, native):
    """configure_file() of src/definitions.h / src/costmatrix (CMakeLists.txt:19-33, 79-81)."""
    out = template.replace("@EF@", ef)
    out = out.replace("@COST@", ("const float COST[]%s;" % cost) if cost else "")
    flags = {"REDUCEMAX": reducemax, "PROTECTED": protected, "NATIVE": native}
    out = re.sub(r"#cmakedefine (\w+) 1",
                 lambda m: ("#define %s 1" % m.group(1)) if flags.get(m.group(1)) else
                 ("/* #undef %s */" % m.group(1)), out)
    return out


def extract_decode(ppi_cc):
    """decode_rule .. end of decode() from src/ppi.cc (lines 106-182)."""
    src = open(ppi_cc).read()
    start = src.index("t_rule* decode_rule(")
    dec = src.index("int decode(", start)
    depth, i, opened = 0, src.index("{", dec), False
    while True:
        if src[i] == "{":
            depth += 1
            opened = True
        elif src[i] == "}":
            depth -= 1
            if opened and depth == 0:
                break
        i += 1
    return src[start:i + 1] + "\n"


def extract_read(main_cc):
    """read() of src/main.cc (lines 32-119): PPI's CSV dataset reader."""
    src = open(main_cc).read()
    start = src.index("int read( const std::string& dataset")
    depth, i = 0, src.index("{", start)
    while True:   # braces outside comments and string / character literals
        c = src[i]
        if src.startswith("//", i):
            i = src.index("\n", i)
            continue
        if src.startswith("/*", i):
            i = src.index("*/", i) + 2
            continue
        if c in "\"'":
            j = i + 1
            while src[j] != c:
                j += 2 if src[j] == "\\" else 1
            i = j + 1
            continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                break
        i += 1
    return src[start:i + 1] + "\n"


def build_csv(ref):
    """libref_csv.so: the reference's read() + oracle/ref_csv_driver.cc."""
    os.makedirs(OUT, exist_ok=True)
    open(os.path.join(OUT, "csv_extract.inc"), "w").write(
        extract_read(os.path.join(ref, "src", "main.cc")))
    run(["g++", "-O2", "-fPIC", "-shared", "-w", "-std=c++17", "-I", OUT,
         "-I", os.path.join(ref, "src", "util"), os.path.join(HERE, "ref_csv_driver.cc"),
         "-o", os.path.join(OUT, "libref_csv.so")])


def run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout


def build_one(ref, name, spec):
    gram, ef, cost, rmax, prot, native, mps = spec
    d = os.path.join(OUT, name)
    inc = os.path.join(d, "include")
    os.makedirs(inc, exist_ok=True)
    gpath = grammar_path(ref, gram)
    run([sys.executable, os.path.join(ref, "script", "read_grammar.py"), "-o", inc, "-g", gpath,
         "-i", os.path.join(ref, "src", "interpreter", "interpreter_core"),
         "-p", os.path.join(ref, "src", "interpreter", "ppi_individual_print_function")])
    defs = configure(open(os.path.join(ref, "src", "definitions.h")).read(), ef, None, rmax, prot,
                     native)
    if ef == GUARDED_COST_EF:
        defs = GUARD_HELPER + defs
    open(os.path.join(inc, "definitions.h"), "w").write(defs)
    open(os.path.join(inc, "costmatrix"), "w").write(
        configure(open(os.path.join(ref, "src", "costmatrix")).read(), ef, cost, rmax, prot, native))
    shutil.copy(os.path.join(ref, "src", "interpreter", "functions.h"), os.path.join(inc, "functions.h"))
    open(os.path.join(d, "decode_extract.inc"), "w").write(
        extract_decode(os.path.join(ref, "src", "ppi.cc")))
    dflags = ["-DPROTECTED"] * prot + ["-DNATIVE"] * native
    common = ["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w"] + dflags
    interp = os.path.join(ref, "src", "interpreter")
    run(common + ["-std=c++17", "-I", inc, "-iquote", interp,
                  os.path.join(interp, "sequential.cc"), os.path.join(HERE, "ref_seq_driver.cc"),
                  "-o", os.path.join(d, "libref_seq.so")])
    run(common + ["-std=c++20", "-I", inc, "-I", HERE,
                  '-DACCEL_CL_PATH="%s"' % os.path.join(interp, "accelerator.cl"),
                  "-DMAX_PHENOTYPE_SIZE=%d" % mps, "-DMAX_STACK_SIZE=%d" % mps,
                  os.path.join(HERE, "ref_cl_driver.cc"), "-o", os.path.join(d, "libref_cl.so"),
                  "-lpthread"])
    run(common + ["-std=c++17", "-I", inc, "-I", d, os.path.join(HERE, "ref_decode_driver.cc"),
                  "-o", os.path.join(d, "libref_decode.so")])
    sym = open(os.path.join(inc, "symbol")).read()
    enum = re.search(r"typedef enum \{(.*?)\} Symbol;", sym, re.S).group(1)
    return name, {"grammar": gpath, "ef": ef, "cost": cost, "reduce_max": rmax, "protected": prot,
                  "native": native, "max_size": mps, "symbol_enum": " ".join(enum.split()),
                  "not_using_t_const": "NOT_USING_T_CONST" in sym}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=reference_root())
    ap.add_argument("--only", nargs="*")
    a = ap.parse_args()
    if not os.path.isdir(os.path.join(a.ref, "src", "interpreter")):
        print("reference tree not found at %s; nothing built" % a.ref)
        return 0
    names = a.only or list(CONFIGS)
    os.makedirs(OUT, exist_ok=True)
    man_path = os.path.join(OUT, "manifest.json")
    manifest = json.load(open(man_path)) if os.path.exists(man_path) else {}
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        csv = ex.submit(build_csv, a.ref)
        for name, info in ex.map(lambda n: build_one(a.ref, n, CONFIGS[n]), names):
            manifest[name] = info
        csv.result()
    json.dump(manifest, open(man_path, "w"), indent=1)
    print("built %d reference configurations into %s" % (len(names), OUT))
    return 0


if __name__ == "__main__":
    sys.exit(main())
