"""Drop-in for the reference's `eob.new_Dormand_horiz.DOPR853` (eob/new_Dormand_horiz.py:219-778).

The batched DOPR853 driver with the reference's interface and semantics: the
12 stages of a step run as one fused launch (eob_dopr853_steps), then the error
norm and step controller, accept/scatter, dense output, stopping rule, and the
fixed-step mode used by the fine pass.  Arrays are torch CUDA tensors.

This is the reference-shaped, step-by-step path; SEOBNRv4PHM's waveform calls
run the persistent integrator of libeobgb300 instead (one launch per batch).
"""
from __future__ import annotations

import torch

from . import pydopr853


class DOPR853:
    def __init__(self, ode, stopping_criterion=None, tmax=1e300, max_step=int(1e6), use_gpu=True,
                 read_out_to_cpu=False):
        if not use_gpu:
            raise ValueError("this implementation runs on the GPU only (no CPU fallback)")
        self.ode = ode
        self.stopping_criterion = stopping_criterion
        self.tmax, self.max_step = tmax, max_step
        self.use_gpu = True
        self.read_out_to_cpu = read_out_to_cpu
        self.stop_info = None

    def integrate(self, condBound, argsData, hInit=None, step_num=None, denseOutput=None, denseOutputLoc=None,
                  fix_step=False):
        dev = torch.device("cuda")
        if denseOutput is None:
            solOld = torch.as_tensor(condBound, dtype=torch.float64, device=dev).clone()
            nODE, numSys = solOld.shape
            denseOutput = torch.zeros((self.max_step, nODE, numSys), dtype=torch.float64, device=dev)
            denseOutputLoc = torch.zeros((self.max_step, numSys), dtype=torch.float64, device=dev)
            step_num = torch.zeros(numSys, dtype=torch.int64, device=dev)
            x = torch.zeros(numSys, dtype=torch.float64, device=dev)
            denseOutput[0] = solOld
            denseOutputLoc[0] = x
        else:
            max_steps, nODE, numSys = denseOutput.shape
            step_num = torch.as_tensor(step_num, device=dev).to(torch.int64)
            cols = torch.arange(numSys, device=dev)
            x = denseOutputLoc[step_num, cols].clone()
            solOld = denseOutput[step_num, :, cols].T.contiguous()
        if self.stopping_criterion is not None and hasattr(self.stopping_criterion, "setup"):
            self.stopping_criterion.setup(numSys)
        additionalArgs = torch.as_tensor(argsData, dtype=torch.float64, device=dev)
        if hInit is None:
            hInit = 0.01
        hInit_orig = torch.full((numSys,), float(hInit), dtype=torch.float64, device=dev)
        h = hInit_orig.clone()
        errOld = torch.full((numSys,), 1e-4, dtype=torch.float64, device=dev)
        previousReject = torch.zeros(numSys, dtype=torch.bool, device=dev)
        active = torch.ones(numSys, dtype=torch.bool, device=dev)
        # the reference initialises its stop flags to True (new_Dormand_horiz.py:582): a system whose
        # first attempt is rejected stops there
        stop = torch.ones(numSys, dtype=torch.bool, device=dev)
        self.stop_info = torch.zeros(numSys, dtype=torch.int64, device=dev)
        nargs = nODE
        while True:
            idx = torch.nonzero(active).flatten()
            n = int(idx.numel())
            if n == 0:
                break
            xT = x[idx].contiguous()
            hT = h[idx].contiguous()
            solT = solOld[:, idx].contiguous()
            solNewT = torch.zeros_like(solT)
            errOldT = errOld[idx].contiguous()
            prevT = previousReject[idx].to(torch.uint8).contiguous()
            addT = additionalArgs[:, idx].contiguous()
            ks = [torch.zeros((nODE, n), dtype=torch.float64, device=dev) for _ in range(10)]
            xc = torch.zeros(n, dtype=torch.float64, device=dev)
            arg = torch.zeros((nODE, n), dtype=torch.float64, device=dev)
            ak = torch.zeros((nODE, n), dtype=torch.float64, device=dev)
            err = torch.zeros(n, dtype=torch.float64, device=dev)
            flag = torch.zeros(n, dtype=torch.uint8, device=dev)
            index_here = idx.to(torch.int32)
            pydopr853.dormandPrinceSteps(xT, xc, solT, hT, arg, addT, *ks, ak, nargs, n, additionalArgs.shape[0],
                                         self.ode, index_here)
            k1, k2, k3, k4, k5, k6, k7, k8, k9, k10 = ks
            pydopr853.error(err, solT, solNewT, hT, k1, k2, k3, k6, k7, k8, k9, k10, n, nargs)
            hOld = hT.clone()
            pydopr853.controllerSuccess(flag, err, errOldT, prevT, hT, xT, n, nargs)
            ok = flag.bool()
            if fix_step:
                rej = idx[~ok]
                if rej.numel():
                    hInit_orig[rej] /= 2
                hT = hInit_orig[idx].clone()
            solT[:, ok] = solNewT[:, ok]
            xT[ok] = xT[ok] + hOld[ok]
            x[idx] = xT
            h[idx] = hT
            solOld[:, idx] = solT
            errOld[idx] = errOldT
            previousReject[idx] = prevT.bool()
            upd = idx[ok]
            step_num[upd] += 1
            if upd.numel():
                denseOutput[step_num[upd], :, upd] = solOld[:, upd].T
                denseOutputLoc[step_num[upd], upd] = x[upd]
                if self.stopping_criterion is not None:
                    st = torch.as_tensor(self.stopping_criterion(step_num, solOld[:, upd], additionalArgs[:, upd],
                                                                 upd), device=dev)
                else:
                    st = torch.zeros(upd.numel(), dtype=torch.int64, device=dev)
                self.stop_info[upd] = st.to(torch.int64)
                stop[upd] = st.to(torch.bool)
            active &= ~((x >= self.tmax) | (step_num >= self.max_step - 1) | stop)
        if self.stopping_criterion is not None and hasattr(self.stopping_criterion, "reset"):
            self.stopping_criterion.reset()
        return denseOutputLoc, denseOutput, step_num
