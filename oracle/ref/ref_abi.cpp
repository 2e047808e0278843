/* extern "C" probe ABI over the reference's host-compiled kernels.
 *
 * Test infrastructure only.  Built by oracle/ref/build_ref.sh together with
 * the reference's own sources (src/EOB.cu, src/DOPR853.cu, and lines 1-308
 * of src/interpolate.cu, compiled in place as host C++) into
 * oracle/_ref/libeobref.so.  Each entry point forwards to the reference
 * function named in its comment, unchanged, so that ctypes can drive the
 * reference's CPU path from tests/golden/make_golden.py.
 */
#include "EOB.hh"
#include "DOPR853.hh"
#include "interpolate.hh"
#include <cstring>

extern "C" {

/* src/EOB.cu:127 evaluate_Ham_align_AD_wrap */
void ref_evaluate_H(double *out, double *r, double *phi, double *pr, double *pphi,
                    double *m1, double *m2, double *chi1, double *chi2,
                    double K, double d5, double dSO, double dSS, int n)
{
    evaluate_Ham_align_AD_wrap(out, r, phi, pr, pphi, m1, m2, chi1, chi2, K, d5, dSO, dSS, n);
}

/* src/EOB.cu:242 grad_Ham_align_AD_wrap */
void ref_grad_H(double *arg, double *grad, double *add, int n) { grad_Ham_align_AD_wrap(arg, grad, add, n); }

/* src/EOB.cu:391 hessian_Ham_align_AD_wrap */
void ref_hessian_H(double *arg, double *hess, double *add, int n) { hessian_Ham_align_AD_wrap(arg, hess, add, n); }

/* src/EOB.cu:3033 root_find_all_wrap */
void ref_root_find_all(double *xOut, double *x0In, double *argsIn, double *addIn, int max_iter, double err,
                       int numBinAll, int n, int num_args, int num_add_args)
{
    root_find_all_wrap(xOut, x0In, argsIn, addIn, max_iter, err, numBinAll, n, num_args, num_add_args);
}

/* src/EOB.cu:3343 SEOBNRv5 */
void *ref_eob_create(void) { return new SEOBNRv5(); }
void ref_eob_destroy(void *p) { delete (SEOBNRv5 *)p; }

/* src/EOB.cu:3355 SEOBNRv5::update_information; prefixes are interleaved re/im */
void ref_eob_update(void *p, double *m1, double *m2, double *eta, double *tplspin, double *chiS, double *chiA,
                    int use_hm, int n, double *prefixes)
{
    ((SEOBNRv5 *)p)->update_information(m1, m2, eta, tplspin, chiS, chiA, use_hm, n, (cmplx *)prefixes);
}

/* src/EOB.cu:3376 SEOBNRv5::deallocate_information */
void ref_eob_dealloc(void *p) { ((SEOBNRv5 *)p)->deallocate_information(); }

int ref_coeffs_ndouble(void) { return (int)(sizeof(FacWaveformCoeffs) / sizeof(double)); }

/* raw copy of the per-binary FacWaveformCoeffs (include/EOB.hh:17-362) */
void ref_eob_coeffs(void *p, double *out, int n)
{
    std::memcpy(out, ((SEOBNRv5 *)p)->hCoeffs, sizeof(FacWaveformCoeffs) * (size_t)n);
}

/* src/EOB.cu:3486 SEOBNRv5::ODE_Ham_align_AD_wrap */
void ref_eob_ode(void *p, double *x, double *arg, double *k, double *add, int n, int *idx)
{
    ((SEOBNRv5 *)p)->ODE_Ham_align_AD_wrap(x, arg, k, add, n, idx);
}

/* src/EOB.cu:3385 SEOBNRv5::RR_force_wrap */
void ref_eob_rr_force(void *p, double *force, double *grad, double *args, double *add, int n, int *idx)
{
    ((SEOBNRv5 *)p)->RR_force_wrap(force, grad, args, add, n, idx);
}

/* src/EOB.cu:3398 SEOBNRv5::root_find_scalar_all_wrap */
void ref_eob_root_find_scalar_all(void *p, double *pr_res, double *bounds, double *argsIn, double *addIn,
                                  int max_iter, double err, int numBinAll, int num_args, int num_add_args)
{
    ((SEOBNRv5 *)p)->root_find_scalar_all_wrap(pr_res, bounds, argsIn, addIn, max_iter, err, numBinAll,
                                               num_args, num_add_args);
}

/* src/EOB.cu:3410 SEOBNRv5::IC_diss_wrap */
void ref_eob_ic_diss(void *p, double *out, double *pr, double *args, double *add, double *grad,
                     double *grad_tmp, double *hess, double *force, int n)
{
    ((SEOBNRv5 *)p)->IC_diss_wrap(out, pr, args, add, grad, grad_tmp, hess, force, n);
}

/* src/EOB.cu:3423 SEOBNRv5::EOBGetSpinFactorizedWaveform_wrap; out and prefix are interleaved re/im */
void ref_eob_waveform(void *p, double *out, double *r, double *phi, double *pr, double *pphi, double *v,
                      double *Hreal, double *eta, double *vPhi, int l, int m, double *prefix, double h22_calib,
                      int numSys, int traj_length, int *idx)
{
    ((SEOBNRv5 *)p)->EOBGetSpinFactorizedWaveform_wrap((cmplx *)out, r, phi, pr, pphi, v, Hreal, eta, vPhi, l, m,
                                                      (cmplx *)prefix, h22_calib, numSys, traj_length, idx);
}

/* src/DOPR853.cu:357 dormandPrinceSteps_wrap */
void ref_dopr_steps(double *x, double *xCurrent, double *solOld, double *h, double *arg, double *add,
                    double *k1, double *k2, double *k3, double *k4, double *k5, double *k6, double *k7,
                    double *k8, double *k9, double *k10, double *ak, int nargs, int numEq, int num_add_args,
                    void *ode, int *idx)
{
    dormandPrinceSteps_wrap(x, xCurrent, solOld, h, arg, add, k1, k2, k3, k4, k5, k6, k7, k8, k9, k10, ak, nargs,
                            numEq, num_add_args, (SEOBNRv5 *)ode, idx);
}

/* src/DOPR853.cu:620 error_wrap */
void ref_dopr_error(double *err, double *solOld, double *solNew, double *h, double *k1, double *k2, double *k3,
                    double *k6, double *k7, double *k8, double *k9, double *k10, int numEq, int nargs)
{
    error_wrap(err, solOld, solNew, h, k1, k2, k3, k6, k7, k8, k9, k10, numEq, nargs);
}

/* src/DOPR853.cu:764 controllerSuccess_wrap; bool arrays are one byte per entry */
void ref_dopr_controller(unsigned char *flag, double *err, double *errOld, unsigned char *prevReject, double *h,
                         double *x, int numEq, int nargs)
{
    controllerSuccess_wrap((bool *)flag, err, errOld, (bool *)prevReject, h, x, numEq, nargs);
}

/* src/interpolate.cu:269 interpolate_TD */
void ref_interpolate_TD(double *t, double *y, double *B, double *ud, double *diag, double *ld, int *lengths,
                        int numBinAll, int nsubs)
{
    interpolate_TD(t, y, B, ud, diag, ld, lengths, numBinAll, nsubs);
}

} /* extern "C" */
