"""Host programs reach the device in compact form (upload.cu): only each
row's used prefix travels, and the device rows are rebuilt from it.  The host
entry points must give the same fitness and best index as the device entry
points fed the full rows, whatever the padding holds and whatever the sizes
are (sizes outside [1, max_size] mean an empty program)."""
import numpy as np
import pytest

from helpers import assert_bitexact, load_golden, make_evaluator


def _garbage_padding(d, rng):
    ph = d["phenotype"].copy()
    ep = d["ephemeral"].copy()
    sz = d["size"].copy()
    for i in range(len(sz)):
        k = max(0, min(int(sz[i]), ph.shape[1]))
        ph[i, k:] = rng.integers(-5, 1 << 20, ph.shape[1] - k)
        ep[i, k:] = rng.normal(0, 1e6, ph.shape[1] - k).astype(np.float32)
    # sizes the translator treats as empty programs
    sz[::17] = 0
    sz[5::23] = -3
    sz[9::29] = ph.shape[1] + 1
    return ph, ep, sz


@pytest.mark.gpu
@pytest.mark.parametrize("name,strategy", [("random", "PDP"), ("allops", "PP"), ("cfg5", "DP")])
def test_host_upload_equals_device_rows(gpu_lib, name, strategy):
    import torch
    d = load_golden(name)
    ph, ep, sz = _garbage_padding(d, np.random.default_rng(3))
    ev = make_evaluator(d, strategy, 0, "fast")
    fit_h, best_h = ev.evaluate(ph, ep, sz, 1e-3)
    dev = torch.device("cuda", 0)
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (ph, ep, sz)]
    fit_d = torch.empty(len(sz), dtype=torch.float32, device=dev)
    best_d = torch.empty(1, dtype=torch.int32, device=dev)
    ev.evaluate_device(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), len(sz), 1e-3,
                       fit_d.data_ptr(), best_d.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize()
    assert_bitexact(fit_h, fit_d.cpu().numpy(), name)
    assert int(best_h) == int(best_d.cpu().numpy()[0])
    # a second, smaller population through the same staging area
    k = len(sz) // 3
    fit_k, _ = ev.evaluate(ph[:k], ep[:k], sz[:k], 1e-3)
    assert_bitexact(fit_k, fit_d.cpu().numpy()[:k], name + " prefix")
    ev.close()


@pytest.mark.gpu
def test_batch_host_upload_equals_device_rows(gpu_lib):
    """One fixture's programs as three populations (PDP, PP, DP) of a batch."""
    import torch
    import ppi_gpu
    d = load_golden("random")
    ph, ep, sz = _garbage_padding(d, np.random.default_rng(5))
    cuts = np.array_split(np.arange(len(sz)), 3)
    pops = [dict(rows=d["rows"], n=len(c), strategy=s, error_fn=d["ef"],
                 reduce_max=bool(d["reduce_max"]), protected=bool(d["protected"]))
            for c, s in zip(cuts, ("PDP", "PP", "DP"))]
    be = ppi_gpu.BatchEvaluator(d["symtab"], d["max_size"], pops, "fast")
    fit_h, best_h = be.evaluate(ph, ep, sz)
    dev = torch.device("cuda", 0)
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (ph, ep, sz)]
    fit_d = torch.empty(len(sz), dtype=torch.float32, device=dev)
    best_d = torch.empty(len(pops), dtype=torch.int32, device=dev)
    be.evaluate_device(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), fit_d.data_ptr(),
                       best_d.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize()
    assert_bitexact(fit_h, fit_d.cpu().numpy(), "batch")
    assert np.array_equal(best_h, best_d.cpu().numpy())
    be.close()
