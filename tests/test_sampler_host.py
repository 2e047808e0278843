"""Host logic of the sampler-facing interface (eobgpu_gb300/sampler.py): the
eleven-parameter layout and transforms of the reference's sampling script
(test_pe_eob.py:22, 57-62), its priors with periodic dimensions (:81-100)
and its start-point recipe (:154-170)."""
import numpy as np

from eobgpu_gb300 import sampler as s


def test_transform_matches_the_reference_layout():
    mt, q, inc, beta = 60.0, 2.5, np.pi / 3, np.pi / 5
    x = np.array([mt, q, 1e-4, 1e-4, 100.0, 0.8, np.cos(inc), np.pi / 4, np.sin(beta), np.pi / 6, 2.0])
    y = s.transform(x)
    assert y.shape == (11, 1)
    np.testing.assert_allclose(y[:, 0], [mt * q / (1 + q), mt / (1 + q), 1e-4, 1e-4, 100.0 * 1e6 * s.PC_SI, 0.8, inc,
                                         np.pi / 4, beta, np.pi / 6, 2.0], rtol=1e-15)
    # leading dimensions flatten in C order
    X = np.stack([x, x * 1.01])[None, :, None, :]
    Y = s.transform(X)
    assert Y.shape == (11, 2)
    np.testing.assert_allclose(Y[:, 1], s.transform(x * 1.01)[:, 0])


def test_prior_box_and_periodic_wrap():
    p = s.UniformPrior.reference(Tobs=6.0)
    rng = np.random.default_rng(0)
    x = p.rvs((4, 5), rng)
    assert x.shape == (4, 5, 11)
    assert np.all(np.isfinite(p.logpdf(x)))
    np.testing.assert_allclose(p.logpdf(x), -np.sum(np.log(p.high - p.low)))
    bad = x.copy()
    bad[0, 0, 1] = 7.0  # q above its box
    assert p.logpdf(bad)[0, 0] == -np.inf and np.isfinite(p.logpdf(bad)[0, 1])
    w = x.copy()
    w[..., 5] += 4 * np.pi
    w[..., 9] -= 3 * np.pi
    np.testing.assert_allclose(p.wrap(w)[..., [5, 9]], x[..., [5, 9]], atol=1e-12)


def test_start_points_recipe():
    mean = np.array([60.0, 2.5, 1e-4, 1e-4, 100.0, 0.8, 0.5, 0.785, 0.588, 0.524, 2.0])
    x = s.start_points(mean, ntemps=3, nwalkers=7, factor=0.02, rng=np.random.default_rng(1))
    assert x.shape == (3, 7, 1, 11)
    assert np.all(np.abs(x[..., 6]) <= 0.99) and np.all(np.abs(x[..., 8]) <= 0.99)
    assert np.all((x[..., 5] >= 0) & (x[..., 5] < 2 * np.pi))
    assert np.all(np.abs(x[..., 0] / mean[0] - 1) < 0.02 * 1e-3 * 6)


class _FakeBBH:
    """Records the batches it is asked for; lnL = -m1 (so values are traceable)."""

    def __init__(self):
        self.calls = []

    def get_ll(self, params, **kw):
        self.calls.append((len(params[0]), kw))
        return -np.asarray(params[0])


def test_vectorized_likelihood_batches_and_prior():
    fake = _FakeBBH()
    prior = s.UniformPrior.reference(Tobs=6.0)
    like = s.VectorizedLikelihood(fake, {"Tobs": 6.0, "return_type": "detector_fd"}, prior=prior, max_batch=4)
    x = prior.rvs((2, 5), np.random.default_rng(2))
    x[1, 3, 1] = 9.0  # outside the prior: not evaluated
    ll = like(x)
    assert ll.shape == (2, 5)
    assert ll[1, 3] == -np.inf
    assert [n for n, _ in fake.calls] == [4, 4, 1]
    assert all("return_type" not in kw and kw["Tobs"] == 6.0 for _, kw in fake.calls)
    m1 = s.transform(x)[0].reshape(2, 5)
    ok = np.isfinite(ll)
    np.testing.assert_allclose(ll[ok], -m1[ok])
    lp = like.log_prob(x)
    np.testing.assert_allclose(lp[ok], ll[ok] + prior.logpdf(x)[ok])
