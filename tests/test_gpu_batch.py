"""Batched evaluation: many populations with different datasets, strategies,
lane counts, error functions and reductions in one persistent launch.  Every
fitness and best index must be bit-identical to evaluating each population
alone with the plain evaluator (and, in parity math, to the oracle)."""
import numpy as np
import pytest

from helpers import ProgramGen, assert_bitexact, expected_best, load_golden

pytestmark = pytest.mark.gpu


def _population(d, rng, nlin, nfeat, n, ef, wide=False, **kw):
    X = rng.normal(0, 2, (nlin, nfeat)).astype(np.float32)
    if ef in ("misclass", "cost"):
        y = rng.integers(0, 4, nlin).astype(np.float32)
    else:
        y = rng.normal(0, 2, nlin).astype(np.float32)
    rows = np.concatenate([X, y[:, None]], 1)
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.random(int(k)) for k in rng.integers(0, 50, n - 3)]
    progs += [gen.full(7), gen.full(3)[:5]]          # generic path; malformed
    progs += [[]]                                     # size 0
    if wide:
        # sums of many distinct columns: tiles beyond the main pass's rows
        G = gen.G
        add, attr = gen.by_op[G.OP["ADD"]][0], gen.by_op[G.OP["ATTRIBUTE"]][0]
        for k in (20, 35, 50, min(nfeat, 70)):
            cols = rng.permutation(nfeat)[:k]
            progs[rng.integers(len(progs))] = [(add, 0.0)] * (k - 1) + [(attr, float(c)) for c in cols]
    rng.shuffle(progs)
    p = dict(rows=rows, n=n, error_fn=ef, programs=progs, **kw)
    if ef == "cost":
        c = rng.uniform(0.5, 2.0, (4, 4)).astype(np.float32)
        np.fill_diagonal(c, 0.0)
        p["cost"] = c
    return p


def _mixed(d, seed=0):
    rng = np.random.default_rng(seed)
    return [
        _population(d, rng, 777, 3, 60, "abs", strategy="PDP", protected=1),
        _population(d, rng, 1, 1, 7, "squared", strategy="PP"),
        _population(d, rng, 2049, 5, 41, "misclass", strategy="DP", lanes=48),
        _population(d, rng, 130, 2, 33, "abs", strategy="PDP", lanes=100, reduce_max=1),
        _population(d, rng, 3000, 4, 90, "cost", strategy="PDP"),
        _population(d, rng, 1024, 1, 5, "squared", strategy="DP", lanes=0, protected=1),
        _population(d, rng, 5000, 6, 120, "abs", strategy="PDP", lanes=1024),
        _population(d, rng, 300, 2, 3, "abs", strategy="PP", reduce_max=1),
        _population(d, rng, 2500, 80, 50, "squared", wide=True, strategy="PDP", protected=1),
        _population(d, rng, 700, 60, 20, "abs", wide=True, strategy="DP", lanes=32),
    ]


def _stack(pops, max_size):
    ph, ep, sz = [], [], []
    for p in pops:
        a, b, c = ProgramGen.rows(p["programs"], max_size)
        ph.append(a)
        ep.append(b)
        sz.append(c)
    return np.concatenate(ph), np.concatenate(ep), np.concatenate(sz)


def _plain(d, p, ph, ep, sz, max_size, math, alpha):
    import ppi_gpu
    ev = ppi_gpu.Evaluator(d["symtab"], max_size, len(sz), p.get("strategy", "PDP"),
                           p.get("lanes", 0), p["error_fn"], p.get("cost"),
                           bool(p.get("reduce_max", 0)), bool(p.get("protected", 0)), math)
    ev.set_dataset(p["rows"])
    f, best = ev.evaluate(ph, ep, sz, alpha)
    lanes = ev.lanes
    ev.close()
    return f, best, lanes


@pytest.mark.parametrize("math", ["parity", "fast"])
@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_batch_matches_plain_evaluations(gpu_lib, oracle_lib, math, flags):
    import ppi_gpu
    d = load_golden("allops")
    max_size = 160
    pops = _mixed(d, seed=flags)
    ph, ep, sz = _stack(pops, max_size)
    alpha = np.array([1e-6 * (k + 1) for k in range(len(pops))], np.float32)
    be = ppi_gpu.BatchEvaluator(d["symtab"], max_size, pops, math)
    be.set_alpha(alpha)
    for rep in range(2):                           # second run replays the graph
        fit, best = be.evaluate(ph, ep, sz, flags)
        begin = 0
        for k, p in enumerate(pops):
            sl = slice(begin, begin + p["n"])
            f, b, lanes = _plain(d, p, ph[sl], ep[sl], sz[sl], max_size, math, alpha[k])
            assert_bitexact(fit[sl], f, "population %d (%s, rep %d)" % (k, p.get("strategy"), rep))
            assert best[k] == b, (k, best[k], b)
            if math == "parity":
                ref = oracle_lib.Oracle(p["rows"], d["symtab"], p["error_fn"], p.get("cost"),
                                        p.get("reduce_max", 0), p.get("protected", 0)).evaluate(
                    ph[sl], ep[sl], sz[sl], p.get("strategy", "PDP"), lanes, alpha[k])
                assert_bitexact(fit[sl], ref, "oracle, population %d" % k)
                o = oracle_lib.Oracle(p["rows"], d["symtab"], p["error_fn"], p.get("cost"),
                                      p.get("reduce_max", 0), p.get("protected", 0))
                assert best[k] == expected_best(oracle_lib, o, ph[sl], ep[sl], sz[sl],
                                                p.get("strategy", "PDP"), lanes, alpha[k]), k
            begin += p["n"]
    block, grid, rows, tune = be.shape()
    assert block in (64, 128) and grid >= 1
    if flags & ppi_gpu.BATCH_AUTOTUNE:
        assert max(tune) > 0.0
    assert be.last_kernel_ms() > 0.0
    be.close()


def test_batch_device_entry_with_graph_on_a_stream(gpu_lib):
    """ppi_batch_evaluate_device on a caller's stream, graph captured once and
    replayed; new buffers re-capture."""
    import torch
    import ppi_gpu
    d = load_golden("cfg2")
    max_size = 128
    rng = np.random.default_rng(21)
    pops = [_population(d, rng, nlin, 1, n, "abs", strategy="PDP", protected=1)
            for nlin, n in ((5000, 40), (100, 200), (40000, 17))]
    ph, ep, sz = _stack(pops, max_size)
    host = ppi_gpu.BatchEvaluator(d["symtab"], max_size, pops, "fast")
    f_ref, b_ref = host.evaluate(ph, ep, sz, 0)
    be = ppi_gpu.BatchEvaluator(d["symtab"], max_size, pops, "fast")
    s = torch.cuda.Stream()
    outs = []
    for copy in range(2):
        dph = torch.from_numpy(ph).cuda()
        dep = torch.from_numpy(ep).cuda()
        dsz = torch.from_numpy(sz).cuda()
        dfit = torch.full((len(sz),), float("nan"), device="cuda")
        dbest = torch.full((len(pops),), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        for _ in range(3):
            be.evaluate_device(dph.data_ptr(), dep.data_ptr(), dsz.data_ptr(), dfit.data_ptr(),
                               dbest.data_ptr(), s.cuda_stream, ppi_gpu.BATCH_GRAPH)
        s.synchronize()
        outs.append((dfit.cpu().numpy(), dbest.cpu().numpy()))
    for f, b in outs:
        assert_bitexact(f, f_ref, "device batch")
        assert (b == b_ref).all()
    host.close()
    be.close()


def test_batch_rejects_bad_populations(gpu_lib):
    import ppi_gpu
    d = load_golden("cfg2")
    rows = np.zeros((10, 2), np.float32)
    with pytest.raises(ppi_gpu.PpiGpuError):
        ppi_gpu.BatchEvaluator(d["symtab"], 64, [dict(rows=rows, n=0, error_fn="abs")])
    with pytest.raises(ppi_gpu.PpiGpuError):
        ppi_gpu.BatchEvaluator(d["symtab"], 64, [dict(rows=rows, n=4, error_fn="cost")])
    with pytest.raises(ppi_gpu.PpiGpuError):      # DP lanes above the widest tile
        ppi_gpu.BatchEvaluator(d["symtab"], 64, [dict(rows=np.zeros((5000, 2), np.float32), n=4,
                                                      error_fn="abs", strategy="DP", lanes=4000)])


def test_uneven_workload_programs_are_well_formed_and_match(gpu_lib):
    """A reduced uneven batch from the workload generator (random valid trees
    of geometric length): the batch equals per-population evaluation."""
    import ppi_gpu
    from ppi_gpu import workloads as W
    g, pops = W.uneven_batch(seed=3, n_pops=6, pop_range=(20, 400), rec_range=(100, 20000))
    sv, so, sl = g.symbol_table_arrays()
    ph = np.concatenate([p["phenotype"] for p in pops])
    ep = np.concatenate([p["ephemeral"] for p in pops])
    sz = np.concatenate([p["size"] for p in pops])
    be = ppi_gpu.BatchEvaluator((sv, so, sl), ph.shape[1], pops, "fast")
    fit, best = be.evaluate(ph, ep, sz, ppi_gpu.BATCH_AUTOTUNE)
    begin = 0
    for k, p in enumerate(pops):
        ev = ppi_gpu.Evaluator((sv, so, sl), ph.shape[1], p["n"], "PDP", 0, "abs", None, False, True,
                               "fast")
        ev.set_dataset(p["rows"])
        f, b = ev.evaluate(p["phenotype"], p["ephemeral"], p["size"])
        assert_bitexact(fit[begin:begin + p["n"]], f, "uneven population %d" % k)
        assert best[k] == b
        begin += p["n"]
        ev.close()
    be.close()
