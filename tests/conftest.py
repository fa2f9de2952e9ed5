import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.lib()
    return O


def load_golden(name):
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"), allow_pickle=False))


def grad_scale(ctx64, cls, n, lmax):
    """s_l = T_l sqrt(2 / (2l + 1)), with T_l = tr(C^-1 dC/dC_l) the gradient of a zero map (FP64
    path).  The gradient g_l = T_l - a^T (dC/dC_l) a (a = C^-1 d) is the difference of two terms of
    size T_l; over data realisations its standard deviation is sigma_l = sqrt(2 tr((C^-1 dC/dC_l)^2)),
    and because dC/dC_l = B_l^2 sum_m Y_lm Y_lm^T has rank <= 2l + 1, Cauchy-Schwarz gives
    sigma_l >= s_l.  s_l is therefore a lower bound on the gradient's own statistical scatter, the
    floor below which a relative bar on g_l (which can vanish by cancellation) stops meaning anything."""
    import numpy as np
    T = ctx64.loglike(cls, np.zeros(n), grad=True)["grad"]
    ell = np.arange(lmax + 1)
    return np.asarray(T) * np.sqrt(2.0 / (2 * ell + 1))


def assert_grad_close(g, g_ref, s, rel, what=""):
    """Every component l >= 2: |g - g_ref| <= rel * max(|g_ref|, s_l) (s from grad_scale).
    Returns the worst ratio of error to bound."""
    import numpy as np
    g, g_ref, s = (np.atleast_2d(np.asarray(a)) for a in (g, g_ref, s))
    err = np.abs(g[:, 2:] - g_ref[:, 2:])
    bound = rel * np.maximum(np.abs(g_ref[:, 2:]), s[:, 2:])
    worst = float((err / bound).max())
    assert worst <= 1.0, (what, worst, np.unravel_index(np.argmax(err / bound), err.shape))
    return worst
