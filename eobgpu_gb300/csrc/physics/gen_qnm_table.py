"""Generate qnm_table.h: fundamental (n = 0) quasi-normal-mode frequencies of
a Kerr black hole, M omega_lm(a) for (l, m) = (2,2), (2,1), (3,3), (4,4),
(5,5) and spins -0.99 <= a <= 0.99, for the ringdown of the waveform (the
reference takes them from lalsimulation's tabulated QNMs).  The grid is
uniform in x = sqrt(1 - a): near a = 1 the frequencies go as sqrt(1 - a), so
they are smooth in x and a four-point interpolation stays accurate there.

Method: Leaver's continued fractions (E. W. Leaver, Proc. R. Soc. Lond. A
402, 285 (1985)) for gravitational perturbations (s = -2), in units 2M = 1:
the radial three-term recurrence (his eqs. 25-26) and the angular one of the
spin-weighted spheroidal harmonics (eqs. 20-21), both required to terminate
(continued fraction equal to zero); for each omega the angular separation
constant A is solved for first, then omega by a complex secant iteration.
Each mode is followed from its Schwarzschild value (a = 0) to both ends of
the spin range, so that a < 0 gives the mode of the counter-rotating hole.
Convention: e^{-i omega t}, Im(omega) < 0.

    python gen_qnm_table.py > qnm_table.h
"""
from __future__ import annotations

import sys

import numpy as np

S = -2
MODES = [(2, 2), (2, 1), (3, 3), (4, 4), (5, 5)]
X_MIN, X_MAX, DX = 0.1, 1.411, 0.001   # x = sqrt(1 - a): a from 0.99 down to -0.990921


def _cf(alpha, beta, gamma, n_terms):
    """beta_0 - alpha_0 gamma_1 / (beta_1 - alpha_1 gamma_2 / (beta_2 - ...)),
    evaluated from the bottom."""
    v = beta(n_terms)
    for n in range(n_terms - 1, -1, -1):
        v = beta(n) - alpha(n) * gamma(n + 1) / v
    return v


def angular_cf(A, w, a, m, n_terms=200):
    c = a * w
    k1, k2 = 0.5 * abs(m - S), 0.5 * abs(m + S)
    return _cf(lambda k: -2.0 * (k + 1) * (k + 2 * k1 + 1),
               lambda k: (k * (k - 1) + 2 * k * (k1 + k2 + 1 - 2 * c)
                          - (2 * c * (2 * k1 + S + 1) - (k1 + k2) * (k1 + k2 + 1)) - (c * c + S * (S + 1) + A)),
               lambda k: 2 * c * (k + k1 + k2 + S), n_terms)


def radial_cf(w, A, a, m, n_terms=400):
    b = np.sqrt(1 - 4 * a * a)
    x = w / 2 - a * m
    c0 = 1 - S - 1j * w - 2j / b * x
    c1 = -4 + 2j * w * (2 + b) + 4j / b * x
    c2 = S + 3 - 3j * w - 2j / b * x
    c3 = w * w * (4 + 2 * b - a * a) - 2 * a * m * w - S - 1 + (2 + b) * 1j * w - A + (4 * w + 2j) / b * x
    c4 = S + 1 - 2 * w * w - (2 * S + 3) * 1j * w - (4 * w + 2j) / b * x
    return _cf(lambda n: n * n + (c0 + 1) * n + c0,
               lambda n: -2 * n * n + (c1 + 2) * n + c3,
               lambda n: n * n + (c2 - 3) * n + c4 - c2 + 2, n_terms)


def _secant(f, x, tol=1e-14, iters=80):
    x0, x1 = x, x * (1 + 1e-5) + 1e-7
    f0, f1 = f(x0), f(x1)
    for _ in range(iters):
        if f1 == f0:
            return x1
        x2 = x1 - f1 * (x1 - x0) / (f1 - f0)
        if abs(x2 - x1) < tol * max(1.0, abs(x2)):
            return x2
        x0, f0, x1, f1 = x1, f1, x2, f(x2)
    raise RuntimeError("QNM iteration did not converge")


def qnm(l, m, a_spin, w_guess, A_guess):
    """(M omega, A) of the (l, m, n = 0) mode at spin a_spin (M = 1), from a
    nearby guess."""
    a = 0.5 * a_spin
    state = {"A": A_guess}

    def F(w2):
        state["A"] = _secant(lambda A: angular_cf(A, w2, a, m), state["A"])
        return radial_cf(w2, state["A"], a, m)

    w2 = _secant(F, 2.0 * w_guess)
    return w2 / 2.0, state["A"]


SCHWARZSCHILD_GUESS = {2: 0.3737 - 0.0890j, 3: 0.5994 - 0.0927j, 4: 0.8092 - 0.0942j, 5: 1.0123 - 0.0949j}


def qnm_at(l, m, a_spin):
    """M omega of the (l, m, 0) mode at any spin, followed from a = 0 (no
    table): steps uniform in sqrt(1 - a), 0.01 apart, so that they shrink
    where the frequencies change fast near a = 1."""
    w, A = qnm(l, m, 0.0, SCHWARZSCHILD_GUESS[l], l * (l + 1) - 2.0)
    x1 = np.sqrt(1.0 - a_spin)
    n = int(np.ceil(abs(x1 - 1.0) / 0.01))
    for x in np.linspace(1.0, x1, n + 1)[1:]:
        w, A = qnm(l, m, 1.0 - x * x, w, A)
    return w


def table(l, m, spins):
    """M omega at the given spins, followed from a = 0 outwards."""
    out = np.zeros(len(spins), dtype=complex)
    i0 = int(np.argmin(np.abs(spins)))
    w, A = qnm(l, m, spins[i0], SCHWARZSCHILD_GUESS[l], l * (l + 1) - 2.0)
    out[i0] = w
    for step in (1, -1):
        wp, Ap = w, A
        i = i0 + step
        while 0 <= i < len(spins):
            wp, Ap = qnm(l, m, spins[i], wp, Ap)
            out[i] = wp
            i += step
    return out


def main():
    n = int(round((X_MAX - X_MIN) / DX)) + 1
    x = X_MIN + DX * np.arange(n)
    spins = 1.0 - x * x
    rows = {lm: table(*lm, spins) for lm in MODES}
    w = sys.stdout.write
    w("// Generated by gen_qnm_table.py (Leaver's continued fractions); do not edit.  Fundamental\n")
    w("// Kerr quasi-normal modes M omega_lm(a), e^{-i omega t} convention, on a grid uniform in\n")
    w("// x = sqrt(1 - a): node j at x = kQnmX0 + j kQnmDx.\n")
    w("#pragma once\n\nnamespace eob {\n\n")
    w(f"constexpr double kQnmX0 = {X_MIN!r};\nconstexpr double kQnmDx = {DX!r};\nconstexpr int kQnmN = {n};\n\n")
    w("}  // namespace eob\n\n")
    w("// [mode: (2,2), (2,1), (3,3), (4,4), (5,5)][node][re, im]\n")
    w("#define EOB_QNM_INIT \\\n    { \\\n")
    for lm in MODES:
        w("        { \\\n")
        vals = rows[lm]
        for j in range(0, n, 2):
            w("            " + " ".join(f"{{{v.real.hex()}, {v.imag.hex()}}}," for v in vals[j:j + 2]) + " \\\n")
        w("        }, \\\n")
    w("    }\n")


if __name__ == "__main__":
    main()
