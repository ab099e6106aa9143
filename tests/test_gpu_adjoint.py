"""GPU constant adjoint (ppi_gpu_constant_gradient): d(fitness)/d(constants)
against the oracle's FP64 adjoint (itself checked against FP64 central
differences on the CPU), edge cases, a torch.autograd.Function wrapper, and
gradient-based constant refinement re-judged by the plain evaluator."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLT_MAX = np.float32(3.4028235e38)


def _setup(ef="squared", math="fast", nlin=3000, population=300, seed=3):
    import ppi_gpu
    from ppi_gpu import workloads as W
    g, rows, ph, ep, sz = W.adjoint(seed=seed, nlin=nlin, population=population)
    sym = g.symbol_table_arrays()
    ev = ppi_gpu.Evaluator(sym, ph.shape[1], population, "PDP", 0, ef, None, False, True, math)
    ev.set_dataset(rows)
    return g, rows, ph, ep, sz, ev


def _in_float_range(fit, ref):
    """Programs whose fitness and reference gradients are well inside float
    range: beyond ~1e30 the float reverse sweep's intermediate products can
    overflow where the double one does not (a fitness of 1e35 is no fit)."""
    return (fit < 1e30) & np.all(np.isfinite(ref), 1) & np.all(np.abs(ref) < 1e30, 1)


def _rel(ref, got, rows_ok):
    """Relative error of each nonzero reference component of the selected
    programs; the denominator has a floor at 1e-6 of the program's largest
    gradient."""
    a, b = ref[rows_ok], got[rows_ok].astype(np.float64)
    scale = np.maximum(np.abs(a).max(1, keepdims=True), 1e-12)
    m = a != 0
    return (np.abs(a - b) / np.maximum(np.abs(a), 1e-6 * scale))[m]


@pytest.mark.parametrize("ef", ["squared", "abs"])
def test_parity_gradient_is_the_float_functions_gradient(gpu_lib, oracle_lib, ef):
    """In parity math the GPU forward values are the reference's float values;
    its gradient must then equal the gradient of that float function
    (oracle: float forward, double reverse) to float rounding of the sweep."""
    g, rows, ph, ep, sz, ev = _setup(ef, "parity")
    grad = ev.constant_gradient(ph, ep, sz)
    fit, _ = ev.evaluate(ph, ep, sz)
    o = oracle_lib.Oracle(rows, g.symbol_table_arrays(), ef, None, False, True, False)
    _, gff = o.adjoint64(ph, ep.astype(np.float64), sz, float_forward=True)
    ok = _in_float_range(fit, gff)
    rel = _rel(gff, grad, ok)
    assert rel.size > 500
    assert np.all(np.isfinite(rel))
    assert (rel <= 1e-5).mean() >= 0.999, np.sort(rel)[-5:]


@pytest.mark.parametrize("ef", ["squared", "abs"])
@pytest.mark.parametrize("math", ["fast", "parity"])
def test_gradient_matches_fp64_adjoint(gpu_lib, oracle_lib, ef, math):
    """Against the FP64 adjoint (checked against FP64 central differences on
    the CPU): within 1e-4 relative wherever the float evaluation itself is
    well conditioned, i.e. the gradients of the float function and of the
    double function agree to 1e-5.  Elsewhere (divisions by ~1e-20, values
    near float overflow, protected thresholds) float and double evaluate
    different functions and only the fraction is recorded."""
    g, rows, ph, ep, sz, ev = _setup(ef, math)
    grad = ev.constant_gradient(ph, ep, sz)
    fit, _ = ev.evaluate(ph, ep, sz)
    o = oracle_lib.Oracle(rows, g.symbol_table_arrays(), ef, None, False, True, False)
    f64, g64 = o.adjoint64(ph, ep.astype(np.float64), sz)
    _, gff = o.adjoint64(ph, ep.astype(np.float64), sz, float_forward=True)
    ok = _in_float_range(fit, gff) & np.all(np.isfinite(g64), 1) & np.all(np.abs(g64) < 1e30, 1)
    cond = np.zeros(len(sz), bool)
    for i in np.flatnonzero(ok):
        r = _rel(g64[i:i + 1], gff[i:i + 1], np.array([True]))
        cond[i] = r.size == 0 or r.max() <= 1e-5
    rel_all = _rel(g64, grad, ok)
    rel_cond = _rel(g64, grad, cond)
    assert rel_cond.size > 400
    assert (rel_cond <= 1e-4).mean() >= 0.995, np.sort(rel_cond)[-5:]
    assert (rel_all <= 1e-4).mean() >= 0.85
    # gradients only at constant tokens
    const = g.symbols["T_CONST"]
    for i in range(len(sz)):
        other = np.ones(ph.shape[1], bool)
        other[:sz[i]] = ph[i, :sz[i]] != const
        assert np.all(grad[i, other] == 0.0) or np.isnan(grad[i]).all()
    # sentinel-fitness programs get zero gradients
    assert np.all(grad[fit == FLT_MAX] == 0.0)


def test_edge_programs(gpu_lib):
    import ppi_gpu
    g, rows, _, _, _, _ = _setup(nlin=500, population=8)
    ev = ppi_gpu.Evaluator(g.symbol_table_arrays(), 128, 8, "PDP", 0, "squared", None, False, True,
                           "fast")
    ev.set_dataset(rows)
    S = g.symbols
    const, attr, add = S["T_CONST"], S["T_ATTRIBUTE"], S["T_ADD"]
    ph = np.zeros((8, 128), np.int32)
    ep = np.zeros((8, 128), np.float32)
    sz = np.zeros(8, np.int32)
    # 0: a lone constant (gradient = mean of 2 (c - y)); 1: size 0;
    # 2: malformed ("+ c"); 3: c + x0
    ph[0, 0], ep[0, 0] = const, 0.5
    sz[0] = 1
    sz[1] = 0
    ph[2, :2] = [add, const]
    sz[2] = 2
    ph[3, :3] = [add, const, attr]
    ep[3, :3] = [0.0, 1.5, 2.0]
    sz[3] = 3
    # 4: 40 constants summed (more than the 32 differentiated)
    ph[4, :79] = [add] * 39 + [const] * 40
    sz[4] = 79
    for i in (5, 6, 7):
        ph[i, 0], ep[i, 0], sz[i] = const, float(i), 1
    grad = ev.constant_gradient(ph, ep, sz)
    y = rows[:, -1].astype(np.float64)
    assert grad[0, 0] == pytest.approx(np.mean(2 * (0.5 - y)), rel=1e-5)
    assert np.all(grad[1] == 0.0)
    assert np.isnan(grad[2]).all()
    x2 = rows[:, 2].astype(np.float64)
    assert grad[3, 1] == pytest.approx(np.mean(2 * (1.5 + x2 - y)), rel=1e-5)
    assert grad[3, 0] == 0.0 and grad[3, 2] == 0.0
    assert np.isnan(grad[4]).all()
    # rejected configurations
    for kw in (dict(error_fn="misclass"), dict(reduce_max=True)):
        ev2 = ppi_gpu.Evaluator(g.symbol_table_arrays(), 128, 8, "PDP", 0,
                                kw.get("error_fn", "squared"), None, kw.get("reduce_max", False),
                                True, "fast")
        ev2.set_dataset(rows)
        with pytest.raises(ppi_gpu.PpiGpuError):
            ev2.constant_gradient(ph, ep, sz)


def test_autograd_function_and_refinement(gpu_lib):
    """A torch.autograd.Function whose forward is the plain evaluator and
    whose backward is the constant adjoint; 5 Adam steps on the constants,
    each re-judged by the plain evaluator, lower the median fitness."""
    torch = pytest.importorskip("torch")
    g, rows, ph, ep, sz, ev = _setup(nlin=5000, population=400, seed=8)
    const = g.symbols["T_CONST"]
    mask = torch.zeros(ph.shape, dtype=torch.bool)
    for i in range(len(sz)):
        mask[i, :sz[i]] = torch.from_numpy(ph[i, :sz[i]] == const)

    class Fitness(torch.autograd.Function):
        @staticmethod
        def forward(ctx, eph):
            e = eph.detach().cpu().numpy()
            fit, _ = ev.evaluate(ph, e, sz)
            ctx.save_for_backward(eph)
            return torch.from_numpy(fit)

        @staticmethod
        def backward(ctx, gout):
            (eph,) = ctx.saved_tensors
            grad = ev.constant_gradient(ph, eph.detach().cpu().numpy(), sz)
            return gout[:, None] * torch.from_numpy(np.nan_to_num(grad))

    c = torch.from_numpy(ep.copy()).requires_grad_(True)
    f0 = Fitness.apply(c)
    f0.sum().backward()
    direct = np.nan_to_num(ev.constant_gradient(ph, ep, sz))
    assert np.array_equal(c.grad.numpy(), direct)
    finite = f0.detach().numpy() < FLT_MAX
    start = np.median(f0.detach().numpy()[finite])
    opt = torch.optim.Adam([c], lr=0.05)
    for _ in range(5):
        opt.zero_grad()
        f = Fitness.apply(c)
        (f * torch.from_numpy(finite.astype(np.float32))).sum().backward()
        c.grad[~mask] = 0.0
        opt.step()
    fit_end, _ = ev.evaluate(ph, c.detach().numpy(), sz)
    end = np.median(fit_end[finite & (fit_end < FLT_MAX)])
    assert end < start


@pytest.mark.parametrize("fixture", ["allops", "allops_prot"])
def test_full_opcode_set_is_the_float_functions_gradient(gpu_lib, oracle_lib, fixture):
    """Every opcode (comparisons, logic, IF_THEN_ELSE, MOD, POW, the
    transcendentals, protected or not) through the full-set kernels, in
    parity math: the gradient of the float function (oracle: float forward,
    double reverse), piecewise-constant opcodes contributing 0."""
    from helpers import ProgramGen, load_golden, make_evaluator, oracle_for
    d = load_golden(fixture)
    rng = np.random.default_rng(11 if fixture == "allops" else 12)
    nfeat = d["rows"].shape[1] - 1
    X = rng.normal(0, 2, (1500, nfeat)).astype(np.float32)
    y = rng.normal(0, 2, 1500).astype(np.float32)
    rows = np.concatenate([X, y[:, None]], 1)
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.random(int(k)) for k in rng.integers(1, 16, 2000)]
    ph, ep, sz = ProgramGen.rows(progs, 64)
    # half of the leaves become constants (the generator draws leaf kinds
    # evenly, and the fixtures name many literals)
    from ppi_gpu import grammar as G
    const = gen.by_op[G.OP["CONST"]][0]
    leafsyms = set(s for op in gen.leaf for s in gen.by_op[op])
    for i in range(len(sz)):
        for k in range(sz[i]):
            if ph[i, k] in leafsyms and rng.random() < 0.5:
                ph[i, k], ep[i, k] = const, np.float32(rng.uniform(-3, 3))
    ev = make_evaluator(d, "PDP", 0, "parity", population=len(sz), max_size=64, rows=rows)
    grad = ev.constant_gradient(ph, ep, sz)
    fit, _ = ev.evaluate(ph, ep, sz)
    o = oracle_for(oracle_lib, d, rows=rows)
    _, gff = o.adjoint64(ph, ep.astype(np.float64), sz, float_forward=True)
    ok = _in_float_range(fit, gff)
    rel = _rel(gff, grad, ok)
    assert rel.size > 200   # most paths pass a piecewise-constant opcode (gradient 0)
    assert (rel <= 1e-5).mean() >= 0.995, np.sort(rel)[-5:]
    assert np.all(grad[fit == FLT_MAX] == 0.0)


def test_record_chunks_and_wide_programs(gpu_lib, oracle_lib):
    """20,000 records (several record chunks per program, the last one
    partial) and programs up to 250 tokens over 64 columns: their rows
    (columns, kept values) exceed what an 8-record tile holds at 4 CTAs per
    SM, and the widest exceed a 128-thread CTA of 4 records, so every launch
    group runs (8 and 4 records per thread, and the narrow-CTA fallback)."""
    import ppi_gpu
    from ppi_gpu import grammar as G
    from ppi_gpu import workloads as W
    from helpers import GRAMMARS
    import os
    rng = np.random.default_rng(21)
    g = G.load(os.path.join(GRAMMARS, "config4_adjoint.bnf"))
    nlin, nfeat = 20000, 64
    X = rng.normal(0, 1, (nlin, nfeat)).astype(np.float32)
    y = (X[:, 0] * X[:, 1] + np.sin(X[:, 2]) + rng.normal(0, 0.05, nlin)).astype(np.float32)
    rows = np.concatenate([X, y[:, None]], 1)
    lengths = np.concatenate([rng.integers(3, 40, 120), rng.integers(150, 251, 120)])
    ph, ep = W.random_programs(rng, lengths, nfeat, g, p_unary=0.1, lo=-2.0, hi=2.0)
    S = g.symbols
    attr, const = S["T_ATTRIBUTE"], S["T_CONST"]
    for i, k in enumerate(lengths):   # leaves: columns, and 1-8 constants
        leaves = np.flatnonzero((ph[i, :k] == attr) | (ph[i, :k] == const))
        ph[i, leaves] = attr
        ep[i, leaves] = rng.integers(0, nfeat, len(leaves)).astype(np.float32)
        pick = rng.choice(leaves, min(len(leaves), int(rng.integers(1, 9))), replace=False)
        ph[i, pick] = const
        ep[i, pick] = rng.uniform(-2.0, 2.0, len(pick)).astype(np.float32)
    max_size = 256
    phf = np.zeros((len(lengths), max_size), np.int32)
    epf = np.zeros((len(lengths), max_size), np.float32)
    phf[:, :ph.shape[1]] = ph
    epf[:, :ep.shape[1]] = ep
    sz = lengths.astype(np.int32)
    ev = ppi_gpu.Evaluator(g.symbol_table_arrays(), max_size, len(sz), "PDP", 0, "squared", None, False,
                           True, "parity")
    ev.set_dataset(rows)
    grad = ev.constant_gradient(phf, epf, sz)
    assert ev.last_launch_count() >= 4   # at least two groups, plus translate and finish
    fit, _ = ev.evaluate(phf, epf, sz)
    o = oracle_lib.Oracle(rows, g.symbol_table_arrays(), "squared", None, False, True, False)
    _, gff = o.adjoint64(phf, epf.astype(np.float64), sz, float_forward=True)
    for part in (lengths < 40, lengths >= 150):
        ok = _in_float_range(fit, gff) & part
        rel = _rel(gff, grad, ok)
        assert rel.size > 100
        assert (rel <= 1e-5).mean() >= 0.995, np.sort(rel)[-5:]
