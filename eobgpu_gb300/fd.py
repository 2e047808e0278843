"""Frequency-domain likelihood of the waveform path on one GPU.

The reference's BBHWaveformTD.get_ll (eob/seobnrv4phm.py:772-823) generates
each binary's mode-summed strain on the uniform grid, takes two real FFTs of
its plus and cross parts, projects them onto every detector with the antenna
patterns and the delay from the geocenter, and reduces the PSD-weighted
residual against the detectors' frequency-domain data.

Here, per batch: the fused waveform path writes the summed strain
h = h_+ + i h_x [B, N] (eob_waveform_strain, zero past each binary's end);
one complex FFT per binary (cuFFT through torch.fft) gives H; the detector
response kernel gives F+, Fx and the delays; one fused kernel
(eob_fd_lnl_from_fft) recovers h~_+ and h~_x from H(f) and H(N - f), projects
and reduces.  Data, PSD and detector geometry stay on the device.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .pipeline import WaveformLikelihood, longest_first

SPEED_OF_LIGHT = 299792458.0


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x) if not torch.is_tensor(x) else x, dtype=dtype).to("cuda").contiguous()


def detector_response(ra, dec, psi, geocent_time, detector_tensors, vertices):
    """(F+, Fx, delay [s]) per (detector, binary), device tensors [nch, B]
    (get_detector_information, eob/seobnrv4phm.py:597-634)."""
    ra, dec, psi, t = (_dev(np.atleast_1d(v) if not torch.is_tensor(v) else v).reshape(-1)
                       for v in (ra, dec, psi, geocent_time))
    D = _dev(detector_tensors).reshape(-1, 9)
    V = _dev(vertices).reshape(-1, 3)
    nch, B = D.shape[0], ra.numel()
    Fp = torch.empty((nch, B), dtype=torch.float64, device="cuda")
    Fx = torch.empty_like(Fp)
    tau = torch.empty_like(Fp)
    _lib.check(_lib.load().eob_detector_response(_p(ra), _p(dec), _p(psi), _p(t), _p(D), _p(V), B, nch, _p(Fp),
                                                 _p(Fx), _p(tau), _stream()), "eob_detector_response")
    return Fp, Fx, tau


def fd_lnl_from_fft(H, data, psd, Fp, Fx, tau, df, start_ind=0, scratch=None):
    """lnL [B] from H [B, N] (complex FFT of the summed strain), data/psd
    [nch, N/2 + 1], F+, Fx, delays [nch, B]."""
    B, N = int(H.shape[0]), int(H.shape[1])
    nch = int(data.shape[0])
    lib = _lib.load()
    need = int(lib.eob_fd_lnl_scratch_bytes(B, N))
    if scratch is None or scratch.numel() < need:
        scratch = torch.empty(max(need, 1), dtype=torch.uint8, device="cuda")
    lnl = torch.empty(B, dtype=torch.float64, device="cuda")
    _lib.check(lib.eob_fd_lnl_from_fft(_p(H), N, int(start_ind), _p(data), _p(psd), _p(Fp), _p(Fx), _p(tau),
                                       float(df), B, nch, _p(scratch), scratch.numel(), _p(lnl), _stream()),
               "eob_fd_lnl_from_fft")
    return lnl


class FDLikelihood:
    """Batched frequency-domain likelihood against fixed detector data.

    data: complex [nch, N/2 + 1] frequency-domain strain per detector; psd:
    [nch, N/2 + 1] (infinite values become 1e300, as the reference does);
    detector_tensors [nch, 3, 3], vertices [nch, 3] (m); N = Tobs x
    sampling_frequency samples of the time-domain template."""

    def __init__(self, data, psd, detector_tensors, vertices, sampling_frequency: float, Tobs: float,
                 modes=((2, 2),), max_batch: int = 1024, max_steps: int = 20000, options=None, start_ind: int = 0):
        self.fs = float(sampling_frequency)
        self.N = int(Tobs * sampling_frequency)
        if self.N % 2:
            raise _lib.EOBError("Tobs x sampling_frequency must be even")
        self.Nf = self.N // 2 + 1
        self.df = 1.0 / (self.N / self.fs)
        self.data = _dev(data, torch.complex128).reshape(-1, self.Nf)
        psd = _dev(psd).reshape(-1, self.Nf).clone()
        psd[torch.isinf(psd)] = 1e300
        self.psd = psd.contiguous()
        self.tensors = _dev(detector_tensors).reshape(-1, 3, 3)
        self.vertices = _dev(vertices).reshape(-1, 3)
        if not (self.data.shape[0] == self.psd.shape[0] == self.tensors.shape[0] == self.vertices.shape[0]):
            raise _lib.EOBError("data, psd, detector tensors and vertices must have one row per detector")
        self.start_ind = int(start_ind)
        self.wl = WaveformLikelihood(max_batch, max_steps, modes, self.N, options=options)
        self.scratch = torch.empty(max(1, int(_lib.load().eob_fd_lnl_scratch_bytes(max_batch, self.N))),
                                   dtype=torch.uint8, device="cuda")

    def strain(self, params, distance):
        """Summed strain [B, N] (plus = real, cross = imaginary) / distance;
        params [B, 5] = (m1, m2, chi1z, chi2z, f0)."""
        P = _dev(params).reshape(-1, 5)
        h, st = self.wl.strain(P, 1.0 / self.fs, self.N, order=longest_first(P))
        self.status = st
        return h / _dev(distance).reshape(-1)[:, None]

    def lnl(self, params, distance, ra, dec, psi, geocent_time):
        h = self.strain(params, distance)
        H = torch.fft.fft(h, dim=-1)
        del h
        Fp, Fx, tau = detector_response(ra, dec, psi, geocent_time, self.tensors, self.vertices)
        return fd_lnl_from_fft(torch.view_as_real(H).contiguous(), self.data, self.psd, Fp, Fx, tau, self.df,
                               self.start_ind, self.scratch)


def split_real_ffts(H):
    """(h~_+, h~_x) [B, N/2 + 1] from the complex FFT H [B, N] of h_+ + i h_x:
    the two real FFTs of the reference (eob/seobnrv4phm.py:736-740)."""
    N = H.shape[-1]
    Nf = N // 2 + 1
    k = torch.arange(Nf, device=H.device)
    z = torch.conj(H[..., (N - k) % N])
    a = H[..., :Nf]
    return 0.5 * (a + z), (a - z) / 2j


class _Geometry:
    def __init__(self, vertex):
        self.vertex = np.asarray(vertex, dtype=np.float64)


class _StrainData:
    def __init__(self, start_time):
        self.start_time = float(start_time)


class Interferometer:
    """The attributes of a bilby interferometer that BBHWaveformTD reads
    (eob/seobnrv4phm.py:521-545), for callers without bilby: detector_tensor
    (3 x 3), geometry.vertex (m, Earth-fixed), strain_data.start_time (GPS s),
    amplitude_spectral_density_array and frequency_domain_strain (N/2 + 1
    bins each)."""

    def __init__(self, detector_tensor, vertex, asd, frequency_domain_strain, start_time=0.0):
        self.detector_tensor = np.asarray(detector_tensor, dtype=np.float64).reshape(3, 3)
        self.geometry = _Geometry(vertex)
        self.strain_data = _StrainData(start_time)
        self.amplitude_spectral_density_array = np.asarray(asd, dtype=np.float64)
        self.frequency_domain_strain = np.asarray(frequency_domain_strain, dtype=np.complex128)

    @staticmethod
    def tensor_from_arms(x_arm, y_arm):
        """Detector tensor of an L-shaped interferometer with unit arm
        directions x, y: (x x^T - y y^T) / 2."""
        x = np.asarray(x_arm, dtype=np.float64)
        y = np.asarray(y_arm, dtype=np.float64)
        x = x / np.linalg.norm(x)
        y = y / np.linalg.norm(y)
        return 0.5 * (np.outer(x, x) - np.outer(y, y))
