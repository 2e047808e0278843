"""Drop-in for the reference's `eob.seobnrv4phm` (eob/seobnrv4phm.py).

Same class names, constructor and call signatures; arrays are torch CUDA
tensors (or numpy arrays, converted on entry).  The waveform call runs the
GB300 path of libeobgb300 (one persistent integrator launch per batch, fused
multipoles, splines and synthesis) instead of the reference's Python-driven
loop; the step-by-step methods (setup_class, get_initial_conditions,
run_trajectory, get_hlms) are kept on the reference-shaped entry points for
callers that use them directly.

Differences from the reference, all deliberate:
* max_step defaults to 20000 trajectory rows (the reference hard-codes 400,
  eob/seobnrv4phm.py:1899, which long binaries exceed);
* each binary's result is what the reference returns for that binary alone
  (its batched stopping rule reads other binaries' frequency history,
  :130-135);
* real and imaginary parts are paired per mode for every number of modes
  (the reference's 0::2 / 1::2 slicing is right only for one mode, :2368);
* NQC corrections and ringdown attachment (needing lalsimulation) are not
  applied: the waveform is the inspiral-plunge part up to the stopping point.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .. import _lib
from .. import fd as fdm
from ..pipeline import WaveformLikelihood, longest_first
from . import pyEOB, pytdinterp
from .new_Dormand_horiz import DOPR853

MTSUN_SI = 4.925491025543576e-06


def _cuda(x, dtype=torch.float64):
    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=dtype)
    return torch.as_tensor(np.asarray(x), dtype=dtype, device="cuda")


def factorial2(n, xp=np):
    """Double factorial through Gamma (eob/seobnrv4phm.py:858-876)."""
    from scipy.special import gamma
    n = np.atleast_1d(n)
    out = np.zeros_like(n, dtype=np.float64)
    odd = (n % 2).astype(bool)
    out[odd] = gamma(n[odd] / 2 + 1) * 2 ** ((n[odd] + 1) / 2) / np.sqrt(np.pi)
    out[~odd] = 2 ** (n[~odd] / 2) * gamma(n[~odd] / 2 + 1)
    return out


def EOBComputeNewtonMultipolePrefixes(m1_in, m2_in, l_in, m_in, xp=np):
    """Newtonian multipole prefactors n_lm c_lm eta, shape (B, nlm)
    (Damour, Iyer & Nagar 2008, eqs. 5-7; eob/seobnrv4phm.py:1703-1776)."""
    m1 = np.atleast_1d(np.asarray(m1_in, dtype=np.float64))[:, None]
    m2 = np.atleast_1d(np.asarray(m2_in, dtype=np.float64))[:, None]
    l = np.atleast_1d(np.asarray(l_in))[None, :]
    m = np.atleast_1d(np.asarray(m_in))[None, :]
    tot = m1 + m2
    eps = (l + m) % 2
    x1, x2 = m1 / tot, m2 / tot
    eta = m1 * m2 / (tot * tot)
    sign = np.where(np.abs(m % 2) == 0, 1, -1)
    test1 = (m1 != m2) | (sign == 1)
    c = (test1 * (np.power(x2, l + eps - 1) + sign * np.power(x1, l + eps - 1))
         + (~test1 & (l == 2)) * -1.0 + (~test1 & (l == 3)) * -1.0 + (~test1 & (l == 4)) * -0.5
         + (~test1 & (l == 5)) * -0.5)
    L = np.broadcast_to(l, c.shape)
    Mm = np.broadcast_to(m, c.shape)
    E = np.broadcast_to(eps, c.shape)
    n = (1j * Mm) ** L
    fac = factorial2(2 * L.ravel() + 1).reshape(L.shape)
    even = E == 0
    with np.errstate(divide="ignore", invalid="ignore"):
        n_even = n * 8.0 * np.pi / fac * np.sqrt(((L + 1) * (L + 2)) / (L * (L - 1.0)))
        mult2 = (2.0 * L + 1) * (L + 2) * (L * L - Mm * Mm) / ((2.0 * L - 1) * (L + 1) * L * (L - 1))
        n_odd = -n * 1j * 16.0 * np.pi / fac * np.sqrt(mult2)
    nn = np.where(even, n_even, n_odd)
    return nn * eta * c


class StoppingCriterion:
    """eob/seobnrv4phm.py:61-150, read for each binary on its own: codes 2 (r < 1),
    3 (r < 6, dr/dt > 0), 4 (r < 6, dpr/dt > 0), 5 (r < 6 and the orbital
    frequency has decreased for the last five steps)."""

    def __init__(self, eob_c_class, max_step, use_gpu=True, read_out_to_cpu=False):
        self.eob_c_class = eob_c_class
        self.max_step = max_step
        self.old_omegas = None

    def setup(self, numSys):
        self.numSys = numSys
        self.old_omegas = torch.zeros((self.max_step, numSys), dtype=torch.float64, device="cuda")

    def reset(self):
        self.old_omegas = None

    def __call__(self, step_num, denseOutput, additionalArgs, index_update):
        if self.old_omegas is None:
            raise ValueError("Must use `setup` attribute before using this method.")
        nargs, n = denseOutput.shape
        args = denseOutput.contiguous().view(-1)
        add = additionalArgs.contiguous().view(-1)
        derivs = torch.zeros(nargs * n, dtype=torch.float64, device="cuda")
        x = torch.zeros(1, dtype=torch.float64, device="cuda")
        self.eob_c_class.ODE_Ham_align_AD(x, args, derivs, add, n, index_update.to(torch.int32).contiguous())
        derivs = derivs.view(nargs, n)
        r, drdt, omega, dprdt = denseOutput[0], derivs[0], derivs[1], derivs[2]
        stop = torch.zeros(n, dtype=torch.int64, device="cuda")
        stop = torch.where(r < 1.0, 2, stop)
        rem = stop == 0
        stop = torch.where(rem & (r < 6.0) & (drdt > 0.0), 3, stop)
        rem = stop == 0
        stop = torch.where(rem & (r < 6.0) & (dprdt > 0.0), 4, stop)
        rem = stop == 0
        steps = step_num[index_update]
        here = rem & (steps > 5)
        if bool(here.any()):
            cols = index_update[here]
            s = steps[here]
            hist = torch.stack([self.old_omegas[s - j, cols] for j in (4, 3, 2, 1)], dim=1)
            c1 = r[here] < 6.0
            c2 = omega[here] < hist[:, 3]
            c3 = torch.all(torch.diff(hist, dim=1) < 0.0, dim=1)
            stop[here] = torch.where(c1 & c2 & c3, 5, 0)
        self.old_omegas[steps, index_update] = omega
        return stop


class CubicSplineInterpolantTD:
    """Batched not-a-knot splines (eob/seobnrv4phm.py:161-386).  x: flat [L][B]
    knot times, y_all: flat [L][nsubs][B] values, lengths[B]."""

    def __init__(self, x, y_all, lengths, nsubs, num_bin_all, use_gpu=True):
        self.lengths = _cuda(lengths, torch.int32)
        self.max_length = int(self.lengths.max().item())
        self.num_bin_all, self.nsubs = num_bin_all, nsubs
        self.x = _cuda(x).contiguous()
        self.y = _cuda(y_all).contiguous()
        n = self.y.numel()
        B = torch.zeros(n, dtype=torch.float64, device="cuda")
        self.c1 = torch.zeros(n, dtype=torch.float64, device="cuda")
        self.c2 = torch.zeros(n, dtype=torch.float64, device="cuda")
        self.c3 = torch.zeros(n, dtype=torch.float64, device="cuda")
        pytdinterp.interpolate_TD_wrap(self.x, self.y, B, self.c1, self.c2, self.c3, self.lengths, num_bin_all, nsubs)
        t = self.x.view(self.max_length, num_bin_all).T.clone()
        rows = torch.arange(self.max_length, device="cuda")[None, :]
        pad = rows >= self.lengths[:, None].long()
        t[pad] = (2.0 * t.max(dim=1).values)[:, None].expand_as(t)[pad]
        self.t_shaped = t

    def _shaped(self, a):
        return a.view(self.max_length, self.nsubs, self.num_bin_all).permute(2, 1, 0)

    # [B][nsubs][L] views, as the reference's properties (eob/seobnrv4phm.py:221-239)
    @property
    def y_shaped(self):
        return self._shaped(self.y)

    @property
    def c1_shaped(self):
        return self._shaped(self.c1)

    @property
    def c2_shaped(self):
        return self._shaped(self.c2)

    @property
    def c3_shaped(self):
        return self._shaped(self.c3)

    @property
    def container(self):
        return [self.x, self.y, self.c1, self.c2, self.c3]

    def __call__(self, tnew, deriv_order=0):
        tnew = _cuda(tnew)
        if tnew.ndim != 2 or tnew.shape[0] != self.num_bin_all:
            raise ValueError("tnew must be 2D with one row per binary")
        inds = torch.searchsorted(self.t_shaped, tnew, right=True) - 1
        inds = torch.where(inds == self.lengths[:, None].long(), inds - 1, inds).clamp(min=0)
        x = tnew - torch.gather(self.t_shaped, 1, inds)
        idx = inds[:, None, :].expand(-1, self.nsubs, -1)
        y = torch.gather(self._shaped(self.y), 2, idx)
        c1 = torch.gather(self._shaped(self.c1), 2, idx)
        c2 = torch.gather(self._shaped(self.c2), 2, idx)
        c3 = torch.gather(self._shaped(self.c3), 2, idx)
        x = x[:, None, :]
        if deriv_order == 0:
            out = y + c1 * x + c2 * x * x + c3 * x * x * x
        elif deriv_order == 1:
            out = c1 + 2 * c2 * x + 3 * c3 * x * x
        elif deriv_order == 2:
            out = 2 * c2 + 6 * c3 * x
        elif deriv_order == 3:
            out = 6 * c3
        else:
            raise ValueError("deriv_order must be within 0 <= deriv_order <= 3.")
        return out.squeeze()


class TDInterp:
    """Mode synthesis from spline containers on a uniform time grid
    (eob/seobnrv4phm.py:389-500) through TDInterp_wrap2: per binary the
    samples before its last knot, each mode spline rotated by e^{-i m phi} and
    summed.  Returns the flat complex template carrier [numBinAll * data_length]."""

    def __init__(self, max_init_len=-1, use_gpu=True):
        if not use_gpu:
            raise ValueError("this implementation runs on the GPU only (no CPU fallback)")
        if max_init_len > 0:
            # as the reference: buffers are not implemented
            raise NotImplementedError
        self.use_buffers = False
        self.template_gen = pytdinterp.TDInterp_wrap2

    @property
    def template_channels(self):
        return [self.template_carrier[i].reshape(self.data_length) for i in range(self.num_bin_all)]

    def __call__(self, dataTime, interp_container, length, data_length, num_modes, ls, ms, numBinAll, dt=1 / 1024):
        self.length, self.num_modes, self.num_bin_all, self.data_length = length, num_modes, numBinAll, data_length
        dataTime = _cuda(dataTime)
        ts = interp_container.t_shaped
        ends = ts.max(dim=1).values
        st = torch.searchsorted(dataTime, torch.zeros_like(ends), right=False)
        et = torch.searchsorted(dataTime, ends.contiguous(), right=False)
        self.lengths = et.to(torch.int32)
        max_length = int(self.lengths.max().item())
        inds = torch.zeros(self.num_bin_all * max_length, dtype=torch.int32, device="cuda")
        old_lengths = interp_container.lengths
        old_length = int(old_lengths.max().item())
        for i in range(self.num_bin_all):
            a, e = int(st[i]), int(et[i])
            inds[i * max_length + a: i * max_length + e] = (
                torch.searchsorted(ts[i].contiguous(), dataTime[a:e].contiguous(), right=True).to(torch.int32) - 1)
        self.template_carrier = torch.zeros(int(data_length * self.num_bin_all), dtype=torch.complex128, device="cuda")
        ls = _cuda(ls, torch.int32)
        ms = _cuda(ms, torch.int32)
        self.template_gen(self.template_carrier, dataTime, ts.contiguous().flatten(),
                          interp_container.y_shaped.contiguous().flatten(),
                          interp_container.c1_shaped.contiguous().flatten(),
                          interp_container.c2_shaped.contiguous().flatten(),
                          interp_container.c3_shaped.contiguous().flatten(), old_length, old_lengths, self.data_length,
                          self.num_bin_all, self.num_modes, ls, ms, inds, self.lengths, max_length)
        return self.template_carrier


def fd_likelihood(hp_fd, hc_fd, data, psd, Fplus, Fcross, time_shift, df, num_bin_all, nchannels, return_complex=False):
    """The likelihood step of BBHWaveformFD.get_ll (eob/seobnrv4phm.py:778-817):
    per-1024-bin partials from all_in_one_likelihood, then
    lnL = -1/2 df 4 sum over blocks and channels.  hp_fd, hc_fd: complex
    [num_bin_all, N]; data, psd: [nchannels, N]; Fplus, Fcross, time_shift:
    [nchannels, num_bin_all] (flattened as the reference does)."""
    hp = _cuda(hp_fd, torch.complex128).reshape(-1)
    hc = _cuda(hc_fd, torch.complex128).reshape(-1)
    d = _cuda(data, torch.complex128).reshape(-1)
    S = _cuda(psd).reshape(-1)
    N = hp.numel() // num_bin_all
    nblk = -(-N // 1024)
    temp = torch.zeros(nblk * num_bin_all * nchannels, dtype=torch.complex128, device="cuda")
    pytdinterp.all_in_one_likelihood(temp, hp, hc, d, S, _cuda(Fplus).reshape(-1), _cuda(Fcross).reshape(-1),
                                     _cuda(time_shift).reshape(-1), df, num_bin_all, nchannels, N)
    like = -1.0 / 2.0 * df * 4.0 * temp.reshape(-1, num_bin_all, nchannels).sum(dim=(0, 2))
    return like if return_complex else like.real


class SEOBNRv4PHM:
    """Aligned-spin SEOBNR waveform generator (eob/seobnrv4phm.py:1845-2726).

    imr (default True, as the reference's __call__): the modes carry the NQC
    correction and the merger-ringdown (compute_full_waveform, :2374-2557);
    imr=False stops at the trajectory's end."""

    allowable_modes_hlms = [(2, 2), (2, 1), (3, 3), (4, 4), (5, 5)]

    def __init__(self, max_init_len=-1, use_gpu=True, ell_max=8, max_step=20000, options=None, imr=True, **kwargs):
        if max_init_len > 0:
            raise NotImplementedError
        self.use_gpu = True
        self.ell_max = ell_max
        lm = [(l, m) for l in range(2, ell_max + 1) for m in range(1, l + 1)]
        self.l_vals = np.array([l for l, _ in lm], dtype=np.int32)
        self.m_vals = np.array([m for _, m in lm], dtype=np.int32)
        self.num_lm = len(lm)
        self.ells_default = np.array([l for l, _ in self.allowable_modes_hlms], dtype=np.int32)
        self.mms_default = np.array([m for _, m in self.allowable_modes_hlms], dtype=np.int32)
        self.max_step = max_step
        self.options = _lib.default_options() if options is None else _lib.EobOptions.from_buffer_copy(options)
        self.options.imr = 1 if imr else 0
        self.eob_c_class = pyEOB.SEOBNRv5Class()
        self.integrator = DOPR853(self.eob_c_class, stopping_criterion=StoppingCriterion(self.eob_c_class, max_step),
                                  tmax=1e7 * 1e6, max_step=max_step)
        self.num_args = 4
        self.num_add_args = 10
        self.num_add_args_total = self.num_add_args + 2 * self.num_lm
        self.K_val = self.d5_val = self.dSO_val = self.dSS_val = self.h22_calib = 0.0
        self._wl = None

    def _sanity_check_modes(self, ells, mms):
        for ell, mm in zip(ells, mms):
            if (int(ell), int(mm)) not in self.allowable_modes_hlms:
                raise ValueError(f"Requested mode [(l,m) = ({ell},{mm})] is not available. "
                                 f"Allowable modes include {self.allowable_modes_hlms}")

    # ---- step-by-step interface (reference-shaped entry points) ----------
    def setup_class(self, m_1_scaled, m_2_scaled, chi_1, chi_2, omega0):
        m1 = _cuda(m_1_scaled)
        m2 = _cuda(m_2_scaled)
        c1, c2 = _cuda(chi_1), _cuda(chi_2)
        B = m1.numel()
        self.num_bin_all = B
        eta = m1 * m2 / (m1 + m2) ** 2
        chiS, chiA = (c1 + c2) / 2, (c1 - c2) / 2
        tpl = (1 - 2 * eta) * chiS + (m1 - m2) / (m1 + m2) * chiA
        pre = EOBComputeNewtonMultipolePrefixes(m1.cpu().numpy(), m2.cpu().numpy(), self.l_vals, self.m_vals).T
        add = torch.zeros((self.num_add_args_total, B), dtype=torch.float64, device="cuda")
        add[0], add[1], add[2], add[3], add[4] = m1, m2, c1, c2, _cuda(omega0)
        add[5], add[6], add[7], add[8], add[9] = self.K_val, self.d5_val, self.dSO_val, self.dSS_val, self.h22_calib
        add[10::2] = _cuda(pre.real)
        add[11::2] = _cuda(pre.imag)
        self.additionalArgs = add
        self.prefixes = _cuda(pre.real) + 1j * _cuda(pre.imag)
        if self.eob_c_class.allocated:
            self.eob_c_class.deallocate_information()
        self.eob_c_class.update_information(m1.contiguous(), m2.contiguous(), eta.contiguous(), tpl.contiguous(),
                                            chiS.contiguous(), chiA.contiguous(), 1, B, None)

    def get_initial_conditions(self, m_1, m_2, chi_1, chi_2, fs=20.0, max_iter=1000, err=1e-12, **kwargs):
        mt = _cuda(m_1) + _cuda(m_2)
        omega0 = fs * (mt * MTSUN_SI * math.pi)
        B = mt.numel()
        r_guess = omega0 ** (-2.0 / 3)
        x0 = torch.stack([r_guess, torch.sqrt(r_guess)]).contiguous()
        xout = torch.zeros_like(x0)
        args = torch.zeros(4 * B, dtype=torch.float64, device="cuda")
        add = self.additionalArgs.contiguous()
        pyEOB.root_find_all(xout, x0, args, add, max_iter, err, B, 2, 4, self.num_add_args_total)
        r0, pphi0 = xout[0], xout[1]
        pr0 = torch.zeros(B, dtype=torch.float64, device="cuda")
        bounds = torch.tensor([[-3e-2], [0.0]], dtype=torch.float64, device="cuda").expand(2, B).contiguous()
        argsIn = torch.zeros((4, B), dtype=torch.float64, device="cuda")
        argsIn[0], argsIn[3] = r0, pphi0
        self.eob_c_class.root_find_scalar_all(pr0, bounds, argsIn.contiguous(), add, max_iter, err, B, 4,
                                              self.num_add_args_total)
        return r0, pphi0, pr0

    def run_trajectory(self, r0, pphi0, pr0, m_1, m_2, chi_1, chi_2, fs=20.0, step_back=10.0, fine_step=0.05,
                       **kwargs):
        """Two-pass trajectory (eob/seobnrv4phm.py:2072-2136) through the step-by-step DOPR853."""
        mt = _cuda(m_1) + _cuda(m_2)
        cond = torch.stack([r0, torch.zeros_like(r0), pr0, pphi0])
        t, traj, num_steps = self.integrator.integrate(cond.clone(), self.additionalArgs)
        B = r0.numel()
        cols = torch.arange(B, device="cuda")
        S = num_steps
        t_stop = t[(S - 1).clamp(min=0), cols]
        idx = torch.argmin(torch.abs(t - (t_stop - step_back)[None, :]), dim=0)
        rows = torch.arange(t.shape[0], device="cuda")[:, None]
        t[rows >= idx[None, :]] = 0.0
        traj[(rows >= idx[None, :])[:, None, :].expand_as(traj)] = 0.0
        t, traj, num_steps = self.integrator.integrate(cond.clone(), self.additionalArgs, step_num=idx - 1,
                                                       denseOutput=traj, denseOutputLoc=t, hInit=fine_step,
                                                       fix_step=True)
        num_steps = (num_steps + 1).to(torch.int32)
        L = int(num_steps.max().item())
        return (t[:L].T * mt[:, None] * MTSUN_SI), traj[:L].permute(2, 1, 0), num_steps

    # ---- the waveform call -------------------------------------------------
    MAX_SAMPLES = 2 ** 22  # uniform-grid samples per binary a call may return

    def _pipeline(self, B):
        if self._wl is None or self._wl.max_batch < B:
            self._wl = WaveformLikelihood(max(B, 1), self.max_step, self.allowable_modes_hlms, self.MAX_SAMPLES,
                                          options=self.options)
        return self._wl

    def __call__(self, m1, m2, chi1z, chi2z, distance, phiRef, modes=None, fs=20.0, nrDeltaT=None,
                 sampling_frequency=16384.0):
        if modes is not None:
            ells = np.asarray([l for l, _ in modes], dtype=np.int32)
            mms = np.asarray([m for _, m in modes], dtype=np.int32)
            self._sanity_check_modes(ells, mms)
        else:
            ells, mms = self.ells_default, self.mms_default
        self.ells, self.mms = ells, mms
        self.num_modes = K = len(ells)
        m1, m2 = _cuda(m1).reshape(-1), _cuda(m2).reshape(-1)
        B = m1.numel()
        self.num_bin_all = B
        fsv = _cuda(fs).expand(B) if np.ndim(fs) == 0 else _cuda(fs)
        params = torch.stack([m1, m2, _cuda(chi1z).reshape(-1), _cuda(chi2z).reshape(-1), fsv.reshape(-1)],
                             dim=1).contiguous()
        dt = 1.0 / sampling_frequency
        wl = self._pipeline(B)
        wl.set_modes(list(zip(ells, mms)))
        wl.prepare(params, dt, order=longest_first(params))
        npts = wl.npts()
        nsteps, _, status, trajs = wl.trajectories()
        self.lengths = torch.as_tensor(nsteps, dtype=torch.int32, device="cuda")
        L = int(nsteps.max())
        mt = (m1 + m2).cpu().numpy()
        t = np.zeros((B, L))
        tr = np.zeros((B, 4, L))
        for b, (tt, yy) in enumerate(trajs):
            t[b, :len(tt)] = tt * mt[b] * MTSUN_SI
            tr[b, :, :len(tt)] = yy.T
        self.t = _cuda(t)
        self.traj = _cuda(tr)
        self.status = status
        nmax = int(npts.max())
        if nmax > wl.max_samples:
            raise _lib.EOBError(f"{nmax} samples exceed the {wl.max_samples} this generator returns")
        out, _ = wl.synth_strain(B, dt, nmax, per_mode=True)
        out = out / _cuda(distance).reshape(-1)[:, None, None]
        return out


class BBHWaveformTD:
    """Mode-summed strain, detector response and likelihood
    (eob/seobnrv4phm.py:503-823).

    bilby_interferometers: objects with bilby's detector_tensor,
    geometry.vertex, strain_data.start_time, amplitude_spectral_density_array
    and frequency_domain_strain (eobgpu_gb300.fd.Interferometer provides them
    without bilby).  return_type "geocenter_td" (sum_lm h_lm on the uniform
    grid, plus = real, cross = imaginary), "geocenter_fd" (its two real FFTs),
    "detector_fd" (projected onto each detector with its delay) or "like"
    (returns None, as the reference); get_ll is the reference's likelihood;
    get_ll_td the white-noise time-domain likelihood of this build.  Each
    binary's template is zero past its own end (the reference's batched
    synthesis holds the last value up to the batch's longest waveform; a
    single-binary call gives zero)."""

    def __init__(self, bilby_interferometers=None, amp_phase_kwargs={}, interp_kwargs={}, use_gpu=True):
        self.amp_phase_gen = SEOBNRv4PHM(**amp_phase_kwargs)
        self.use_gpu = True
        self.bilby_interferometers = bilby_interferometers
        self.num_interp_params = 2
        if bilby_interferometers is not None:
            ifos = list(bilby_interferometers)
            self.detector_tensors = _cuda(np.array([bi.detector_tensor for bi in ifos]))
            self.detector_start_times = _cuda(np.array([bi.strain_data.start_time for bi in ifos]))
            self.detector_vertex = _cuda(np.array([bi.geometry.vertex for bi in ifos]))
            psd = np.array([np.asarray(bi.amplitude_spectral_density_array) ** 2 for bi in ifos]).flatten()
            psd[np.isinf(psd)] = 1e300
            self.psd = _cuda(psd)
            data = np.array([bi.frequency_domain_strain for bi in ifos], dtype=np.complex128)
            self.fd_data_length = data.shape[1]
            self.nChannels = data.shape[0]
            self.data = _cuda(data.flatten(), torch.complex128)
        self._fd = None

    def get_detector_information(self, ra, dec, time, psi):
        """(F+, Fx, delay from the geocenter) [nch, B] (eob/seobnrv4phm.py:597-634)."""
        self._need_ifos()
        return fdm.detector_response(ra, dec, psi, time, self.detector_tensors, self.detector_vertex)

    def _need_ifos(self):
        if self.bilby_interferometers is None:
            raise ValueError("Must provide detector_tensors kwarg.")

    def _templates(self, m1, m2, chi1z, chi2z, distance, modes, fs, N, dt):
        gen = self.amp_phase_gen
        m1 = _cuda(m1).reshape(-1)
        B = m1.numel()
        self.num_bin_all = B
        ells = gen.ells_default if modes is None else np.asarray([l for l, _ in modes], dtype=np.int32)
        mms = gen.mms_default if modes is None else np.asarray([m for _, m in modes], dtype=np.int32)
        self.num_modes = len(ells)
        lm = [(int(l), int(m)) for l, m in zip(ells, mms)]
        key = (B, tuple(lm), N)
        if getattr(self, "_wl_key", None) != key:
            self._wl = WaveformLikelihood(B, gen.max_step, lm, N, options=gen.options)
            self._wl_key = key
        fsv = _cuda(fs).expand(B) if np.ndim(fs) == 0 else _cuda(fs).reshape(-1)
        params = torch.stack([m1, _cuda(m2).reshape(-1), _cuda(chi1z).reshape(-1), _cuda(chi2z).reshape(-1), fsv],
                             dim=1).contiguous()
        h, st = self._wl.strain(params, dt, N, order=longest_first(params))
        self.status = st
        return h / _cuda(distance).reshape(-1)[:, None]

    def __call__(self, m1, m2, chi1z, chi2z, distance, phiRef, inc=None, ra=None, dec=None, psi=None,
                 geocent_time=None, sampling_frequency=1024, Tobs=60.0, modes=None, bufferSize=None, fill=False,
                 fs=20.0, return_type="like", combine_modes=True, bilby_start_ind=0):
        if return_type not in ("geocenter_td", "geocenter_fd", "detector_td", "detector_fd", "like"):
            raise ValueError("return_type must be geocenter_td, geocenter_fd, like, or detector_fd.")
        self.sampling_frequency = sampling_frequency
        self.data_length = N = int(Tobs * sampling_frequency)
        h = self._templates(m1, m2, chi1z, chi2z, distance, modes, fs, N, 1.0 / sampling_frequency)
        if return_type == "geocenter_td":
            return h
        hp, hc = fdm.split_real_ffts(torch.fft.fft(h, dim=-1))
        hp[:, :bilby_start_ind] = 0.0
        hc[:, :bilby_start_ind] = 0.0
        self.templates_out = [hp, hc]
        if return_type == "geocenter_fd":
            return hp, hc
        Fplus, Fcross, time_shift = self.get_detector_information(ra, dec, geocent_time, psi)
        if return_type == "detector_td":
            raise NotImplementedError
        if return_type == "detector_fd":
            f = torch.fft.rfftfreq(N, 1.0 / sampling_frequency, dtype=torch.float64, device="cuda")
            return ((Fplus.T[:, :, None] * hp[:, None, :] + Fcross.T[:, :, None] * hc[:, None, :])
                    * torch.exp(-2j * np.pi * f[None, None, :] * time_shift.T[:, :, None]))
        return None

    def get_ll(self, params, sampling_frequency=1024, return_complex=False, return_cupy=False, Tobs=60.0,
               modes=None, fs=20.0, bilby_start_ind=0, **kwargs):
        """lnL per binary for params = (m1, m2, chi1z, chi2z, distance, phiRef,
        inc, ra, dec, psi, geocent_time), each of length B
        (eob/seobnrv4phm.py:772-823)."""
        self._need_ifos()
        m1, m2, chi1z, chi2z, distance, phiRef, inc, ra, dec, psi, geocent_time = params
        self.sampling_frequency = sampling_frequency
        self.data_length = N = int(Tobs * sampling_frequency)
        if N // 2 + 1 != self.fd_data_length:
            raise ValueError(f"Tobs x sampling_frequency = {N} samples do not match the data's "
                             f"{self.fd_data_length} frequency bins")
        h = self._templates(m1, m2, chi1z, chi2z, distance, modes, fs, N, 1.0 / sampling_frequency)
        H = torch.fft.fft(h, dim=-1)
        del h
        Fplus, Fcross, time_shift = self.get_detector_information(ra, dec, geocent_time, psi)
        df = 1.0 / (N / sampling_frequency)
        like = fdm.fd_lnl_from_fft(torch.view_as_real(H).contiguous(), self.data.view(self.nChannels, -1),
                                   self.psd.view(self.nChannels, -1), Fplus, Fcross, time_shift, df,
                                   bilby_start_ind)
        if return_complex:
            like = like.to(torch.complex128)
        return like if return_cupy else like.cpu().numpy()

    def get_ll_td(self, params, data, amp, sampling_frequency=1024, modes=None, fs=20.0):
        """lnL = -1/2 sum_k (d_k - amp Re sum_lm h_lm(t_k))^2 for params[B, 4] (m1, m2, chi1z, chi2z)."""
        gen = self.amp_phase_gen
        d = _cuda(data)
        P = _cuda(params)
        B = P.shape[0]
        ells = gen.ells_default if modes is None else np.asarray([l for l, _ in modes], dtype=np.int32)
        mms = gen.mms_default if modes is None else np.asarray([m for _, m in modes], dtype=np.int32)
        wl = WaveformLikelihood(B, gen.max_step, [(int(l), int(m)) for l, m in zip(ells, mms)], d.numel(),
                                options=gen.options)
        full = torch.cat([P[:, :4], torch.full((B, 1), float(fs), dtype=torch.float64, device="cuda")],
                         dim=1).contiguous()
        lnl, st = wl.run(full, d.contiguous(), 1.0 / sampling_frequency, float(amp))
        self.status = st
        return lnl
