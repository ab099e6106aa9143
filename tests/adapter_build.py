"""Builds the adapter + integration driver for one configuration (tests only)."""
import os
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(ROOT, "ppi-auto_gb300", "adapter")
DRIVER = os.path.join(ROOT, "tests", "integration", "ppi_driver.cc")


def build_driver(grammar, outdir, ef=None, cost=None, reducemax=False, protected=False,
                 native=False, profiling=False, ppi_headers=None):
    """Generate the headers, compile adapter + driver; returns the executable.

    ppi_headers: (accelerator.h directory, generated-header directory) of a
    PPI build to compile against instead of the compat headers."""
    from ppi_gpu import build as B
    from ppi_gpu import codegen
    gen = os.path.join(outdir, "gen")
    if ppi_headers:
        codegen.write(grammar, gen, map_only=True)
        incs = ["-I", ppi_headers[0], "-I", ppi_headers[1]]
    else:
        codegen.write(grammar, gen, ef=ef, cost=cost, reducemax=reducemax, protected=protected,
                      native=native)
        incs = ["-I", os.path.join(ADAPTER, "compat")]
    exe = os.path.join(outdir, "ppi_driver")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Werror", "-Wno-unused-function"] + incs + [
        "-I", gen, "-I", B.INCLUDE, DRIVER, os.path.join(ADAPTER, "accelerator_cuda.cc"),
        "-o", exe]
    if profiling:
        cmd.insert(1, "-DPROFILING")
    cmd += ["-L", B.OUT, "-lppi_gpu", "-Wl,-rpath," + B.OUT]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("adapter build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return exe


def run_driver(exe, mode, rows, gens, alpha, flags, env=None):
    """gens: list of (phenotype, ephemeral, size); returns per-generation
    (results, best, send_at, recv_at, nimm)."""
    nlin, ncol = rows.shape
    n, mps = gens[0][0].shape
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            np.array([mode, nlin, ncol, n, mps, len(gens)], np.int32).tofile(f)
            np.array([alpha], np.float32).tofile(f)
            np.ascontiguousarray(rows, np.float32).tofile(f)
            for ph, ep, sz in gens:
                np.ascontiguousarray(ph, np.int32).tofile(f)
                np.ascontiguousarray(ep, np.float32).tofile(f)
                np.ascontiguousarray(sz, np.int32).tofile(f)
        e = dict(os.environ)
        e.update(env or {})
        r = subprocess.run([exe, fin, fout] + flags, capture_output=True, text=True, env=e)
        if r.returncode != 0:
            raise RuntimeError("driver failed (%d): %s %s" % (r.returncode, r.stdout, r.stderr))
        raw = np.fromfile(fout, np.float32)
    per = (nlin if mode == 2 else n) + 4
    out = []
    for g in range(len(gens)):
        chunk = raw[g * per:(g + 1) * per]
        res = chunk[:-4]
        tail = chunk[-4:].view(np.int32)
        out.append((res, int(tail[0]), int(tail[1]), int(tail[2]), int(tail[3])))
    return out, r.stdout


# PPI's own sources linked with the adapter (src/main.cc, src/ppi.cc, ...):
# the reference's CMake target minus src/interpreter/accelerator.cc, which the
# adapter replaces (src/CMakeLists.txt:52-56, src/interpreter/CMakeLists.txt).
PPI_SOURCES = ["main.cc", "ppi.cc", "ppp.cc", "common/common.cc", "server/server.cc",
               "client/client.cc", "util/CmdLineParser.cc", "interpreter/sequential.cc"]
POCO_STUB = os.path.join(ROOT, "tests", "integration", "poco_stub")


def build_ppi(ref_src, generated, grammar, outdir):
    """Compile PPI's unchanged sources from the reference tree (ref_src = its
    src/ directory) with the headers its read_grammar.py generated for one
    configuration (`generated`), test-only Poco stand-ins, and the adapter;
    link them against libppi_gpu.so.  Returns the executable."""
    from concurrent.futures import ThreadPoolExecutor
    from ppi_gpu import build as B
    from ppi_gpu import codegen
    gen = os.path.join(outdir, "gen")
    codegen.write(grammar, gen, map_only=True)
    incs = ["-I", POCO_STUB, "-I", generated, "-I", ref_src, "-I", os.path.join(ref_src, "interpreter")]
    # gnu++14: the reference's CMake sets no standard, and ppi.cc's global
    # `data` collides with C++17's std::data under `using namespace std`
    jobs = [(["g++", "-O1", "-std=gnu++14", "-fopenmp", "-w"] + incs +
             ["-c", os.path.join(ref_src, f), "-o", os.path.join(outdir, f.replace("/", "_") + ".o")])
            for f in PPI_SOURCES]
    jobs.append(["g++", "-O1", "-std=c++17", "-Wall", "-Werror", "-I", gen, "-I", generated, "-I", B.INCLUDE,
                 "-I", os.path.join(ref_src, "interpreter"), "-c", os.path.join(ADAPTER, "accelerator_cuda.cc"),
                 "-o", os.path.join(outdir, "accelerator_cuda.o")])
    os.makedirs(outdir, exist_ok=True)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("PPI build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return cmd[-1]
    with ThreadPoolExecutor(8) as ex:
        objs = list(ex.map(run, jobs))
    exe = os.path.join(outdir, "ppi")
    run(["g++", "-fopenmp", "-o", exe] + objs + ["-L", B.OUT, "-lppi_gpu", "-Wl,-rpath," + B.OUT, "-pthread",
                                                 "-o", exe])
    return exe
