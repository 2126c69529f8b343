"""Convergence stop on the FP64 log-likelihood (GPU, C ABI).

mlem_run with loglik_every > 0 and loglik_rel_tol = t ends the run after the
first evaluated iteration whose log-likelihood gained less than t·|L| over the
previous evaluation.  The test derives the expected stopping iteration from a
full run's log-likelihood curve, and checks the iterations reported, the NaN
tail of the curve and that the image equals a plain run of that many
iterations, bit for bit."""
import numpy as np
import pytest

from conftest import problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,every", [("ring2d", 1), ("cyl3d_tiny", 3)])
def test_convergence_stop(pkg, O, name, every):
    p = problem(pkg, O, name)
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    n = 60
    _, ll = m.run(p["g"], n, f0=p["f0"], loglik=True, loglik_every=every)
    evals = np.arange(0, n, every)
    gains = np.diff(ll[evals]) / np.abs(ll[evals[1:]])
    tol = float(np.sort(gains)[len(gains) // 2])  # stops about halfway
    first = int(np.argmax(gains < tol))
    expect = int(evals[first + 1]) + 1
    img, ll2, st = m.run(p["g"], n, f0=p["f0"], loglik=True, stats=True, loglik_every=every, loglik_rel_tol=tol)
    assert st["iterations"] == expect < n
    assert np.all(np.isnan(ll2[expect:]))
    np.testing.assert_array_equal(ll2[:expect][~np.isnan(ll2[:expect])], ll[:expect][~np.isnan(ll[:expect])])
    plain = m.run(p["g"], expect, f0=p["f0"], loglik=True, loglik_every=every)[0]
    assert np.array_equal(img, plain)
    m.close()


def test_convergence_stop_needs_the_log_likelihood(pkg, O):
    p = problem(pkg, O, "ring2d_tiny")
    m = pkg.Matrix.from_csr(p["rp"], p["col"], p["val"], p["cols"])
    for bad in (dict(loglik_rel_tol=1e-6), dict(loglik_every=1, loglik_rel_tol=-1.0)):
        with pytest.raises(pkg.MlemError) as e:
            m.run(p["g"], 5, **bad)
        assert e.value.status == "EINVAL"
    m.close()
