"""The sampler-facing interface on the GPU, following the reference's
parameter-estimation script (test_pe_eob.py): an injection in the
eleven-parameter sampling layout is projected onto three detectors
(return_type "detector_fd") and becomes their data; the vectorised
likelihood then evaluates tempered walkers scattered around it through the
fused frequency-domain get_ll."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOBS, FS = 6.0, 4096.0


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import sampler as s
    from eobgpu_gb300.eob.seobnrv4phm import BBHWaveformTD
    from eobgpu_gb300.fd import Interferometer
    rng = np.random.default_rng(31)
    Nf = int(TOBS * FS) // 2 + 1
    D, V = [], []
    for _ in range(3):
        q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        D.append(Interferometer.tensor_from_arms(q[:, 0], q[:, 1]))
        V.append(6.37e6 * q[:, 2])
    asd = np.full(Nf, 1e-23)
    asd[:20 * int(TOBS)] = np.inf  # below 20 Hz
    empty = [Interferometer(D[c], V[c], asd, np.zeros(Nf, complex)) for c in range(3)]
    inj = np.array([60.0, 2.5, 1e-4, 1e-4, 100.0, 0.8, np.cos(np.pi / 3), np.pi / 4, np.sin(np.pi / 5), np.pi / 6,
                    2.0])
    kw = dict(sampling_frequency=FS, Tobs=TOBS, bufferSize=None, fill=False, bilby_start_ind=0,
              return_type="detector_fd")
    p_in = np.repeat(s.transform(inj), 2, axis=-1)
    data = BBHWaveformTD(empty)(*p_in, **kw)[0].cpu().numpy()
    ifos = [Interferometer(D[c], V[c], asd, data[c]) for c in range(3)]
    bbh = BBHWaveformTD(ifos)
    prior = s.UniformPrior.reference(TOBS)
    like = s.VectorizedLikelihood(bbh, kw, prior=prior)
    return s, bbh, like, prior, inj, kw


def test_injection_is_the_maximum(setup):
    s, bbh, like, prior, inj, kw = setup
    pts = s.start_points(inj, ntemps=2, nwalkers=16, factor=0.5, rng=np.random.default_rng(4))
    ll = like(pts)
    assert ll.shape == (2, 16, 1)
    assert np.all(np.isfinite(ll))
    l0 = like(inj[None, :])[0]
    # the template at the injection reproduces the data
    assert abs(l0) < 1e-9 * np.max(np.abs(ll))
    assert np.all(ll <= l0)
    # the same numbers as a direct get_ll on the transformed walkers
    direct = bbh.get_ll(list(s.transform(pts)), sampling_frequency=FS, Tobs=TOBS)
    np.testing.assert_allclose(ll.ravel(), direct, rtol=1e-12)


def test_walkers_outside_the_prior_are_not_evaluated(setup):
    s, bbh, like, prior, inj, kw = setup
    pts = s.start_points(inj, ntemps=1, nwalkers=4, factor=0.1, rng=np.random.default_rng(5))
    pts[0, 2, 0, 1] = 6.0  # q outside [1, 5]
    ll = like(pts)
    assert ll[0, 2, 0] == -np.inf
    assert np.all(np.isfinite(np.delete(ll.ravel(), 2)))
    lp = like.log_prob(pts)
    assert lp[0, 2, 0] == -np.inf and np.all(np.isfinite(np.delete(lp.ravel(), 2)))
