"""ppi_gpu_evaluate_noalloc -- the entry point for callers that cannot
allocate memory where they evaluate (device memory reserved by another
allocator, a fixed-footprint island process, a loop that must not pay for
cudaMalloc's synchronisation).  It must give the same fitness and best index
as the handle-based entry point, call after call, although every call reuses
the library's one fixed scratch array.  Collected last so that a failure here
comes after every other test has run."""
import ctypes as C

import numpy as np
import pytest

from helpers import ProgramGen, load_golden, make_evaluator

pytestmark = pytest.mark.gpu


def _entry(lib):
    import ppi_gpu
    f = lib.ppi_gpu_evaluate_noalloc
    f.argtypes = [C.POINTER(ppi_gpu._lib.Config), C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_float, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p]
    return f


def _case(d, nprog, nlin, seed, strategy, math):
    rng = np.random.default_rng(seed)
    X = rng.normal(0, 2, (nlin, d["rows"].shape[1] - 1)).astype(np.float32)
    y = rng.normal(0, 2, nlin).astype(np.float32)
    rows = np.concatenate([X, y[:, None]], 1)
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.random(int(k)) for k in rng.integers(0, 50, nprog)]
    ph, ep, sz = ProgramGen.rows(progs, d["max_size"])
    ev = make_evaluator(d, strategy, 0, math, population=nprog, rows=rows)
    fit, best = ev.evaluate(ph, ep, sz, 1e-6)
    return dict(rows=rows, ph=ph, ep=ep, sz=sz, fit=fit, best=best, ev=ev)


def _device(case):
    import torch
    rows = case["rows"]
    nlin, ncol = rows.shape
    ld = (nlin + 3) // 4 * 4
    data = torch.zeros((ncol, ld), dtype=torch.float32, device="cuda")
    data[:, :nlin] = torch.from_numpy(np.ascontiguousarray(rows.T))
    t = {k: torch.from_numpy(case[k]).cuda() for k in ("ph", "ep", "sz")}
    t["fit"] = torch.full((len(case["sz"]),), float("nan"), dtype=torch.float32, device="cuda")
    t["best"] = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    t["status"] = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    return data, ld, t


def _call(f, case, data, ld, t, stream):
    ev = case["ev"]
    cfg = ev._config
    nlin, ncol = case["rows"].shape
    return f(C.byref(cfg), data.data_ptr(), nlin, ncol, ld, t["ph"].data_ptr(),
             t["ep"].data_ptr(), t["sz"].data_ptr(), len(case["sz"]), 1e-6,
             t["fit"].data_ptr(), t["best"].data_ptr(), t["status"].data_ptr(), stream)


@pytest.mark.parametrize("strategy,math", [("PDP", "fast"), ("PP", "parity"), ("DP", "fast")])
def test_noalloc_matches_handle_entry_point(gpu_lib, strategy, math):
    import torch
    f = _entry(gpu_lib)
    d = load_golden("allops")
    big = _case(d, 1500, 3000, 1, strategy, math)
    small = _case(d, 40, 333, 2, strategy, math)
    stream = torch.cuda.current_stream().cuda_stream
    dev_big, dev_small = _device(big), _device(small)
    for case, (data, ld, t) in [(big, dev_big), (small, dev_small), (big, dev_big)]:
        t["fit"].fill_(float("nan"))
        t["best"].fill_(-1)
        t["status"].fill_(-1)
        assert _call(f, case, data, ld, t, stream) == 0
        torch.cuda.synchronize()
        fit = t["fit"].cpu().numpy()
        assert np.array_equal(fit.view(np.int32), case["fit"].view(np.int32))
        assert int(t["best"].cpu()[0]) == case["best"]
        assert int(t["status"].cpu()[0]) == 0   # every program ran, every tile arrived


def test_noalloc_rejects_batches_beyond_the_scratch(gpu_lib):
    import torch
    f = _entry(gpu_lib)
    d = load_golden("cfg2")
    case = _case(d, 8, 100, 3, "PDP", "fast")
    data, ld, t = _device(case)
    cfg = case["ev"]._config
    st = f(C.byref(cfg), data.data_ptr(), 100, 2, ld, t["ph"].data_ptr(), t["ep"].data_ptr(),
           t["sz"].data_ptr(), 100000, 0.0, t["fit"].data_ptr(), t["best"].data_ptr(), None,
           torch.cuda.current_stream().cuda_stream)
    assert st == 4   # PPI_ERR_UNSUPPORTED, nothing launched
