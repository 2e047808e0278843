"""Binaries the integrator gives up on, by the reference's stop rules
(eob/new_Dormand_horiz.py:585-775, the controller of src/DOPR853.cu:674-798):
a pass whose first attempted step is rejected ends there (the reference's stop
flags start true), and a pass that reaches the attempt limit ends there.
Either way the binary gets no template -- its lnL is NaN, so that a sampler
cannot take it for a likelihood -- and its status word says why; a
neighbour in the same batch that finishes is bitwise what it is alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EOB_ST_TRIES, EOB_ST_SHORT, EOB_ST_STOP_REJECT = 8, 16, 32


def _run(rows, N, dt, data, **opts):
    import torch
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    o = _lib.default_options()
    o.lanes_per_binary = 64
    for k, v in opts.items():
        setattr(o, k, v)
    wl = WaveformLikelihood(len(rows), 6000, [(2, 2)], N, options=o)
    P = torch.tensor(rows, dtype=torch.float64, device="cuda")
    D = torch.tensor(data, device="cuda")
    lnl, st = wl.run(P, D, dt, 1.0)
    nsteps = wl.trajectories()[0]
    return lnl.cpu().numpy(), st.cpu().numpy(), nsteps, wl.npts()


@pytest.fixture(scope="module")
def noise():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return np.random.default_rng(11).standard_normal(1 << 15)


def test_rejected_first_step_ends_the_pass(noise, oracle):
    """h_init = 1e6 M: the first attempt's stages leave the Hamiltonian's
    domain, the error estimate is not finite (counted as +inf) and the attempt
    is rejected, so the first pass ends with its initial row: EOB_ST_STOP_REJECT
    | EOB_ST_SHORT, one row, no samples, lnL NaN.  The oracle's integration with the
    same first step also stops its first pass before two rows (its failure
    status)."""
    rows = [[30.0, 20.0, 0.1, -0.2, 20.0], [12.0, 10.0, 0.0, 0.0, 20.0]]
    N, dt = 8192, 1.0 / 1024.0
    data = noise[:N]
    lnl, st, nsteps, npts = _run(rows, N, dt, data, h_init=1e6)
    for b in range(2):
        assert st[b] == EOB_ST_STOP_REJECT | EOB_ST_SHORT, st
        assert nsteps[b] == 1 and npts[b] == 0, (nsteps, npts)
        assert np.isnan(lnl[b]), lnl
    det = oracle.lnl_one(np.array(rows[0]), dt, N, [(2, 2)], data, 1.0, max_step=100, h_init=1e6)
    assert det["status"] == 1, det["status"]


def test_attempt_limit_ends_the_pass(noise):
    """max_tries = 600 attempts per pass: the long binary (20 Msun from
    10 Hz, thousands of steps) ends at the limit with EOB_ST_TRIES |
    EOB_ST_SHORT, no samples and lnL NaN; the short one (150 Msun from 20 Hz) finishes
    below the limit and is bitwise the same as alone with the default limit."""
    rows = [[10.0, 10.0, 0.0, 0.0, 10.0], [90.0, 60.0, 0.3, 0.1, 20.0]]
    N, dt = 1 << 15, 1.0 / 2048.0
    data = noise[:N]
    lnl, st, nsteps, npts = _run(rows, N, dt, data, max_tries=600)
    lnl1, st1, nsteps1, npts1 = _run(rows[1:], N, dt, data)
    assert st[0] == EOB_ST_TRIES | EOB_ST_SHORT, st
    assert npts[0] == 0 and 1 < nsteps[0] <= 601, (nsteps, npts)
    assert np.isnan(lnl[0]), lnl
    assert st[1] == 0 and st1[0] == 0, (st, st1)
    assert nsteps[1] == nsteps1[0] and npts[1] == npts1[0]
    assert lnl[1] == lnl1[0], (lnl[1], lnl1[0])
