"""The oracle's restatement of the reference's time-domain synthesis (TD2,
TD) and frequency-domain likelihood kernels (src/interpolate.cu:323-627) on
cases with closed-form answers."""
import numpy as np

from oracle import td_oracle as T


def _linear_phase_case(B=3, K=2, L=7, seed=0):
    """Per binary: constant mode amplitudes a_k (real), zero imaginary parts,
    orbital phase phi(t) = p0 + w t as cubic splines on knots t_j."""
    rng = np.random.default_rng(seed)
    old_lengths = np.array([L, L - 2, L - 3][:B], dtype=np.int32)
    old_length = int(old_lengths.max())
    nsubs = 2 * K + 1
    ts = np.zeros(B * old_length)
    y = np.zeros(B * nsubs * old_length)
    c1 = np.zeros_like(y)
    amps = rng.uniform(0.5, 2.0, (B, K))
    p0 = rng.uniform(-1, 1, B)
    w = rng.uniform(0.5, 3.0, B)
    for b in range(B):
        olh = int(old_lengths[b])
        tk = np.sort(rng.uniform(0, 10, olh))
        tk[0] = 0.0
        ts[b * old_length: b * old_length + olh] = tk
        base = b * nsubs * old_length
        for k in range(K):
            y[base + k * olh: base + k * olh + olh] = amps[b, k]
        y[base + 2 * K * olh: base + 2 * K * olh + olh] = p0[b] + w[b] * tk
        c1[base + 2 * K * olh: base + 2 * K * olh + olh] = w[b]
    return ts, y, c1, old_lengths, old_length, amps, p0, w


def test_td_interp2_linear_phase():
    B, K = 3, 2
    ts, y, c1, old_lengths, old_length, amps, p0, w = _linear_phase_case(B, K)
    ms = np.array([2, 1])
    data_time = np.linspace(0.0, 9.0, 40)
    max_length = 40
    lengths = np.array([40, 31, 17], dtype=np.int32)
    inds = np.zeros(B * max_length, dtype=np.int32)
    for b in range(B):
        tk = ts[b * old_length: b * old_length + old_lengths[b]]
        inds[b * max_length: b * max_length + lengths[b]] = np.clip(
            np.searchsorted(tk, data_time[:lengths[b]], side="right") - 1, 0, old_lengths[b] - 1)
    out = T.td_interp2(data_time, ts, y, c1, np.zeros_like(y), np.zeros_like(y), old_length, old_lengths, 50, B, K, ms,
                       inds, lengths, max_length)
    for b in range(B):
        t = data_time[:lengths[b]]
        ref = sum(amps[b, k] * np.exp(-1j * ms[k] * (p0[b] + w[b] * t)) for k in range(K))
        np.testing.assert_allclose(out[b * 50: b * 50 + lengths[b]], ref, rtol=0, atol=1e-12)
        assert np.all(out[b * 50 + lengths[b]: (b + 1) * 50] == 0)


def test_td_interp_per_binary_offset():
    """TD writes binary b's samples from element data_length of its output."""
    B, K = 2, 1
    ts, y, c1, old_lengths, old_length, amps, p0, w = _linear_phase_case(B, K, seed=1)
    nsubs = 2 * K + 1
    ms = np.array([2])
    data_time = np.linspace(0.0, 8.0, 25)
    outs, ts_l, y_l, c1_l, inds_l = [], [], [], [], []
    starts = np.array([0, 5], dtype=np.int32)
    lens = np.array([20, 15], dtype=np.int32)
    for b in range(B):
        olh = int(old_lengths[b])
        tk = ts[b * old_length: b * old_length + olh]
        ts_l.append(tk)
        blk = slice(b * nsubs * old_length, b * nsubs * old_length + nsubs * olh)
        y_l.append(y[blk])
        c1_l.append(c1[blk])
        inds_l.append(np.clip(np.searchsorted(tk, data_time[starts[b]: starts[b] + lens[b]], side="right") - 1,
                              0, olh - 1))
        outs.append(np.zeros(30 + lens[b], dtype=np.complex128))
    T.td_interp(outs, data_time, ts_l, y_l, c1_l, [np.zeros_like(a) for a in y_l], [np.zeros_like(a) for a in y_l],
                old_lengths, 30, K, ms, inds_l, starts, lens)
    for b in range(B):
        t = data_time[starts[b]: starts[b] + lens[b]]
        np.testing.assert_allclose(outs[b][30:], amps[b, 0] * np.exp(-2j * (p0[b] + w[b] * t)), rtol=0, atol=1e-12)
        assert np.all(outs[b][:30] == 0)


def test_all_in_one_likelihood_closed_forms():
    rng = np.random.default_rng(2)
    B, nch, N, df = 2, 2, 2500, 0.25
    hp = rng.normal(size=B * N) + 1j * rng.normal(size=B * N)
    hc = rng.normal(size=B * N) + 1j * rng.normal(size=B * N)
    psd = rng.uniform(0.5, 2.0, nch * N)
    Fp, Fc, tau = rng.uniform(-1, 1, nch * B), rng.uniform(-1, 1, nch * B), rng.uniform(-0.02, 0.02, nch * B)
    f = df * np.arange(N)
    # data equal to the projected template of binary 0: its residual vanishes
    data = np.concatenate([(Fp[c * B] * hp[:N] + Fc[c * B] * hc[:N]) * np.exp(-2j * np.pi * f * tau[c * B])
                           for c in range(nch)])
    ts = T.all_in_one_likelihood(hp, hc, data, psd, Fp, Fc, tau, df, B, nch, N)
    nblk = (N + 1023) // 1024
    assert ts.shape == (nblk * B * nch,)
    parts = ts.reshape(nblk, B, nch)
    assert np.max(np.abs(parts[:, 0, :])) < 1e-20 + 1e-12 * np.max(np.abs(parts))
    # zero templates: the block partials are sum |d|^2 / psd over each block
    z = np.zeros_like(hp)
    ts0 = T.all_in_one_likelihood(z, z, data, psd, Fp, Fc, tau, df, B, nch, N).reshape(nblk, B, nch)
    for c in range(nch):
        term = np.abs(data[c * N:(c + 1) * N]) ** 2 / psd[c * N:(c + 1) * N]
        for q in range(nblk):
            np.testing.assert_allclose(ts0[q, :, c].real, term[q * 1024:(q + 1) * 1024].sum(), rtol=1e-13)
    lnl = T.fd_lnl(ts0.reshape(-1), df, B, nch)
    np.testing.assert_allclose(lnl, -2.0 * df * sum(np.sum(np.abs(data[c * N:(c + 1) * N]) ** 2 /
                                                           psd[c * N:(c + 1) * N]) for c in range(nch)), rtol=1e-13)


def test_tdinterp_inputs():
    data_time = np.arange(0.0, 10.0, 0.5)
    t_shaped = np.array([[0.0, 1.0, 3.0, 7.2], [0.0, 2.0, 4.0, 8.0]])
    lens, inds, ml = T.tdinterp_inputs(data_time, t_shaped, np.array([4, 4]))
    np.testing.assert_array_equal(lens, [15, 16])
    assert ml == 16
    np.testing.assert_array_equal(inds[:15], np.searchsorted(t_shaped[0], data_time[:15], side="right") - 1)
