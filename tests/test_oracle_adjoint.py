"""The FP64 constant adjoint of the oracle (the checker of the GPU constant
gradient) against FP64 central finite differences, h = 1e-4.  Protected
functions and abs make the fitness piecewise smooth; a difference quotient
that changes between h and h/10 straddles a kink or jump and says nothing
about the derivative, so only smooth points are compared."""
import numpy as np

from helpers import GRAMMARS  # noqa: F401  (path setup)


def _fd(o, ph, ep, sz, i, k, h):
    e1 = ep[i:i + 1].astype(np.float64).copy()
    e2 = e1.copy()
    e1[0, k] += h
    e2[0, k] -= h
    f1 = o.adjoint64(ph[i:i + 1], e1, sz[i:i + 1])[0][0]
    f2 = o.adjoint64(ph[i:i + 1], e2, sz[i:i + 1])[0][0]
    return (f1 - f2) / (2 * h)


def test_fp64_adjoint_matches_central_differences(oracle_lib):
    from ppi_gpu import workloads as W
    for ef in ("squared", "abs"):
        g, rows, ph, ep, sz = W.adjoint(seed=5, nlin=400, population=60)
        o = oracle_lib.Oracle(rows, g.symbol_table_arrays(), ef, None, False, True, False)
        fit, grad = o.adjoint64(ph, ep.astype(np.float64), sz)
        const = g.symbols["T_CONST"]
        smooth = agree = 0
        # programs whose fitness float can represent (beyond it the float
        # evaluator reports the FLT_MAX sentinel, and a difference quotient
        # of ~1e200 values resolves nothing)
        for i in np.flatnonzero(np.isfinite(fit) & (fit < 1e30)):
            for k in np.flatnonzero(ph[i, :sz[i]] == const):
                a = _fd(o, ph, ep, sz, i, k, 1e-4)
                b = _fd(o, ph, ep, sz, i, k, 1e-5)
                if not (np.isfinite(a) and np.isfinite(b)) or abs(a - b) > 1e-5 * max(abs(a), 1e-6) + 1e-9:
                    continue
                smooth += 1
                agree += abs(a - grad[i, k]) <= 1e-4 * max(abs(a), 1e-6)
        assert smooth > 100
        assert agree >= 0.99 * smooth, (ef, agree, smooth)
        # zero at non-constant tokens
        mask = np.zeros_like(grad, bool)
        for i in range(len(sz)):
            mask[i, :sz[i]] = ph[i, :sz[i]] == const
        assert np.all(grad[~mask & np.isfinite(grad)] == 0.0)


def test_fp64_fitness_is_the_reference_fitness_in_double(oracle_lib):
    """Where both are finite, the FP64 restatement's fitness equals the
    oracle's reference-semantics (float) fitness to float accuracy."""
    from ppi_gpu import workloads as W
    g, rows, ph, ep, sz = W.adjoint(seed=6, nlin=300, population=80)
    o = oracle_lib.Oracle(rows, g.symbol_table_arrays(), "squared", None, False, True, False)
    f64, _ = o.adjoint64(ph, ep.astype(np.float64), sz)
    f32 = o.evaluate(ph, ep, sz, "PP", 1, 0.0)
    ok = np.isfinite(f64) & (f32 < 1e30) & (f64 < 1e30)
    rel = np.abs(f64[ok] - f32[ok]) / np.maximum(np.abs(f64[ok]), 1e-30)
    assert ok.sum() > 50
    assert np.median(rel) < 1e-5
