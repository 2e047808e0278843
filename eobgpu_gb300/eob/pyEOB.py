"""Drop-in for the reference's `eob.pyEOB` extension (src/eob.pyx): same
function and method names, argument order and array layouts, backed by
libeobgb300.so.  Calls are asynchronous on the current torch stream.
"""
from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ._ptr import addr, stream


def _lib_():
    return _lib.load()


def root_find_all(xOut, x0In, argsIn, additionalArgsIn, max_iter, err, numBinAll, n, num_args, num_add_args):
    """src/eob.pyx:51 -> eob_root_find_all (discrete Newton on (r, pphi))."""
    _lib.check(_lib_().eob_root_find_all(addr(xOut), addr(x0In), addr(argsIn), addr(additionalArgsIn), int(max_iter),
                                         float(err), int(numBinAll), int(n), int(num_args), int(num_add_args),
                                         stream()), "root_find_all")


def grad_Ham_align_AD(arg, grad_out, additionalArgs, numSys):
    """src/eob.pyx:61 -> eob_grad_ham."""
    _lib.check(_lib_().eob_grad_ham(addr(arg), addr(grad_out), addr(additionalArgs), int(numSys), stream()),
               "grad_Ham_align_AD")


def hessian_Ham_align_AD(arg, hessian_out, additionalArgs, numSys):
    """src/eob.pyx:70 -> eob_hessian_ham (exact second derivatives)."""
    _lib.check(_lib_().eob_hessian_ham(addr(arg), addr(hessian_out), addr(additionalArgs), int(numSys), stream()),
               "hessian_Ham_align_AD")


def evaluate_Ham_align_AD(out, r, phi, pr, pphi, m_1, m_2, chi_1, chi_2, K, d5, dSO, dSS, numSys):
    """src/eob.pyx:79 -> eob_evaluate_ham."""
    _lib.check(_lib_().eob_evaluate_ham(addr(out), addr(r), addr(phi), addr(pr), addr(pphi), addr(m_1), addr(m_2),
                                        addr(chi_1), addr(chi_2), float(K), float(d5), float(dSO), float(dSS),
                                        int(numSys), stream()), "evaluate_Ham_align_AD")


def IC_cons(res, x, args, additionalArgs, grad_out, numSys):
    """src/eob.pyx:94 -> eob_ic_cons."""
    _lib.check(_lib_().eob_ic_cons(addr(res), addr(x), addr(args), addr(additionalArgs), addr(grad_out), int(numSys),
                                   stream()), "IC_cons")


class SEOBNRv5Class:
    """src/eob.pyx:106: per-binary factorized-waveform coefficients on the device.

    update_information allocates the coefficient tables once per batch (in a
    torch tensor, the caching allocator reuses it); deallocate_information
    releases them.  A second update without deallocation keeps the first tables
    and returns, as the reference does (src/EOB.cu:3357-3362)."""

    def __init__(self, ic_mode: int = 0):
        self._ctx = None
        self.numSys = 0
        self.allocated = False
        self.newtonian_prefixes = None
        self.ic_mode = ic_mode

    def update_information(self, m1, m2, eta, tplspin, chi_S, chi_A, use_hm, numSys, newtonian_prefixes_hlms):
        if self.allocated:
            print("need to run deallocator each step. Exiting.")
            return
        lib = _lib_()
        nbytes = lib.eob_ctx_bytes(int(numSys))
        self._ctx = torch.empty(int(nbytes), dtype=torch.uint8, device="cuda")
        self.numSys = int(numSys)
        self.newtonian_prefixes = newtonian_prefixes_hlms
        _lib.check(lib.eob_ctx_update_information(addr(self._ctx), addr(m1), addr(m2), addr(eta), addr(tplspin),
                                                  addr(chi_S), addr(chi_A), int(use_hm), int(numSys), stream()),
                   "update_information")
        self.allocated = True

    def deallocate_information(self):
        self._ctx = None
        self.allocated = False

    @property
    def conceiled_ptr(self):
        """Address of the coefficient tables (the reference returns its C++ object pointer)."""
        if self._ctx is None:
            raise RuntimeError("update_information has not been called")
        return self._ctx.data_ptr()

    def _need(self):
        if self._ctx is None:
            raise RuntimeError("update_information has not been called")

    def RR_force(self, force_out, grad_out, args, additionalArgs, numSys, hCoeffs_index):
        self._need()
        _lib.check(_lib_().eob_ctx_rr_force(addr(self._ctx), addr(force_out), addr(grad_out), addr(args),
                                            addr(additionalArgs), int(numSys), addr(hCoeffs_index), stream()),
                   "RR_force")

    def ODE_Ham_align_AD(self, x, arg, k, additionalArgs, numSys, hCoeffs_index):
        self._need()
        _lib.check(_lib_().eob_ctx_ode(addr(self._ctx), addr(x), addr(arg), addr(k), addr(additionalArgs),
                                       int(numSys), addr(hCoeffs_index), stream()), "ODE_Ham_align_AD")

    def root_find_scalar_all(self, pr_res, start_bounds, argsIn, additionalArgsIn, max_iter, err, numBinAll,
                             num_args, num_add_args):
        self._need()
        _lib.check(_lib_().eob_ctx_root_find_scalar_all(addr(self._ctx), addr(pr_res), addr(start_bounds),
                                                        addr(argsIn), addr(additionalArgsIn), int(max_iter),
                                                        float(err), int(numBinAll), int(num_args),
                                                        int(num_add_args), int(self.ic_mode), stream()),
                   "root_find_scalar_all")

    def IC_diss(self, out, pr, args, additionalArgs, grad_out, grad_temp_force, hess_out, force_out, numSys):
        """src/EOB.cu:2665-2689 residual rdot(F) - dH/dpr with the exact Hessian."""
        self._need()
        n = int(numSys)
        args.view(4, n)[2] = pr
        grad_Ham_align_AD(args, grad_out, additionalArgs, n)
        hessian_Ham_align_AD(args, hess_out, additionalArgs, n)
        add = additionalArgs.view(-1, n).clone()
        add[4] = grad_out.view(4, n)[3]
        idx = torch.arange(n, dtype=torch.int32, device=args.device)
        self.RR_force(force_out, grad_temp_force, args, add, n, idx)
        h = hess_out.view(16, n)
        dLdr = -h[0] / h[12]
        out.copy_(force_out.view(2, n)[1] / dLdr - grad_out.view(4, n)[2])

    def EOBGetSpinFactorizedWaveform(self, out, r, phi, pr, pphi, v, Hreal, eta, vPhiInput, l, m, newtonian_prefix,
                                     h22_calib, numSys, traj_length, hCoeffs_index):
        self._need()
        _lib.check(_lib_().eob_ctx_waveform(addr(self._ctx), addr(out), addr(r), addr(phi), addr(pr), addr(pphi),
                                            addr(v), addr(Hreal), addr(eta), addr(vPhiInput), int(l), int(m),
                                            addr(newtonian_prefix), float(h22_calib), int(numSys), int(traj_length),
                                            addr(hCoeffs_index), stream()), "EOBGetSpinFactorizedWaveform")

    def compute_hlms(self, hlms, r_arr, phi_arr, pr_arr, L_arr, m1_arr, m2_arr, chi1_arr, chi2_arr, num_steps,
                     num_steps_max, ell_arr_in, mm_arr_in, num_modes, num_bin_all, additionalArgsIn, num_add_args):
        """src/eob.pyx:178 -> eob_ctx_compute_hlms: the modes on the trajectory
        rows, hlms[num_bin_all][num_modes][num_steps_max] (complex128), with the
        Newtonian prefixes given to update_information.  The reference's kernel
        never stores its result (src/EOB.cu:3319); this one does."""
        self._need()
        if self.newtonian_prefixes is None:
            raise RuntimeError("compute_hlms needs the Newtonian prefixes given to update_information")
        _lib.check(_lib_().eob_ctx_compute_hlms(addr(self._ctx), addr(hlms), addr(r_arr), addr(phi_arr),
                                                addr(pr_arr), addr(L_arr), addr(m1_arr), addr(m2_arr),
                                                addr(chi1_arr), addr(chi2_arr), addr(num_steps), int(num_steps_max),
                                                addr(ell_arr_in), addr(mm_arr_in), int(num_modes), int(num_bin_all),
                                                addr(additionalArgsIn), int(num_add_args),
                                                addr(self.newtonian_prefixes), stream()), "compute_hlms")
