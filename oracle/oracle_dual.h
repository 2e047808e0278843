// Forward-mode dual numbers for the oracle: first derivatives (D3) and first
// plus second derivatives (H3) with respect to three variables (r, pr, pphi).
// Test infrastructure: exact derivatives of the oracle's Hamiltonian, used in
// place of the reference's generated derivative expressions
// (src/EOB.cu:203-209, 313-340).
#pragma once
#include <math.h>

namespace oracle {

struct D3 {
    double v, d[3];
    D3() : v(0), d{0, 0, 0} {}
    D3(double x) : v(x), d{0, 0, 0} {}
    static D3 var(double x, int i) { D3 r(x); r.d[i] = 1.0; return r; }
};
inline D3 operator+(const D3 &a, const D3 &b) { D3 r; r.v = a.v + b.v; for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
inline D3 operator-(const D3 &a, const D3 &b) { D3 r; r.v = a.v - b.v; for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
inline D3 operator-(const D3 &a) { D3 r; r.v = -a.v; for (int i = 0; i < 3; ++i) r.d[i] = -a.d[i]; return r; }
inline D3 operator*(const D3 &a, const D3 &b) { D3 r; r.v = a.v * b.v; for (int i = 0; i < 3; ++i) r.d[i] = a.v * b.d[i] + b.v * a.d[i]; return r; }
inline D3 operator/(const D3 &a, const D3 &b)
{
    D3 r; r.v = a.v / b.v;
    for (int i = 0; i < 3; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
    return r;
}
inline D3 operator+(const D3 &a, double b) { D3 r = a; r.v += b; return r; }
inline D3 operator+(double b, const D3 &a) { return a + b; }
inline D3 operator-(const D3 &a, double b) { D3 r = a; r.v -= b; return r; }
inline D3 operator-(double b, const D3 &a) { return D3(b) - a; }
inline D3 operator*(const D3 &a, double b) { D3 r; r.v = a.v * b; for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] * b; return r; }
inline D3 operator*(double b, const D3 &a) { return a * b; }
inline D3 operator/(const D3 &a, double b) { return a * (1.0 / b); }
inline D3 operator/(double b, const D3 &a) { return D3(b) / a; }
inline D3 sqrt(const D3 &a) { D3 r; r.v = ::sqrt(a.v); for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] / (2.0 * r.v); return r; }
inline D3 log(const D3 &a) { D3 r; r.v = ::log(a.v); for (int i = 0; i < 3; ++i) r.d[i] = a.d[i] / a.v; return r; }

// second order: value, gradient g[3], Hessian h[3][3]
struct H3 {
    double v, g[3], h[3][3];
    H3() : v(0) { for (int i = 0; i < 3; ++i) { g[i] = 0; for (int j = 0; j < 3; ++j) h[i][j] = 0; } }
    H3(double x) : H3() { v = x; }
    static H3 var(double x, int i) { H3 r(x); r.g[i] = 1.0; return r; }
};
// apply a scalar function with value f0, first derivative f1, second derivative f2
inline H3 chain(const H3 &a, double f0, double f1, double f2)
{
    H3 r; r.v = f0;
    for (int i = 0; i < 3; ++i) r.g[i] = f1 * a.g[i];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.h[i][j] = f1 * a.h[i][j] + f2 * a.g[i] * a.g[j];
    return r;
}
inline H3 operator+(const H3 &a, const H3 &b)
{
    H3 r; r.v = a.v + b.v;
    for (int i = 0; i < 3; ++i) { r.g[i] = a.g[i] + b.g[i]; for (int j = 0; j < 3; ++j) r.h[i][j] = a.h[i][j] + b.h[i][j]; }
    return r;
}
inline H3 operator-(const H3 &a) { return chain(a, -a.v, -1.0, 0.0); }
inline H3 operator-(const H3 &a, const H3 &b) { return a + (-b); }
inline H3 operator*(const H3 &a, const H3 &b)
{
    H3 r; r.v = a.v * b.v;
    for (int i = 0; i < 3; ++i) r.g[i] = a.v * b.g[i] + b.v * a.g[i];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.h[i][j] = a.v * b.h[i][j] + b.v * a.h[i][j] + a.g[i] * b.g[j] + a.g[j] * b.g[i];
    return r;
}
inline H3 recip(const H3 &a) { const double iv = 1.0 / a.v; return chain(a, iv, -iv * iv, 2.0 * iv * iv * iv); }
inline H3 operator/(const H3 &a, const H3 &b) { return a * recip(b); }
inline H3 operator+(const H3 &a, double b) { H3 r = a; r.v += b; return r; }
inline H3 operator+(double b, const H3 &a) { return a + b; }
inline H3 operator-(const H3 &a, double b) { H3 r = a; r.v -= b; return r; }
inline H3 operator-(double b, const H3 &a) { return H3(b) - a; }
inline H3 operator*(const H3 &a, double b) { return chain(a, a.v * b, b, 0.0); }
inline H3 operator*(double b, const H3 &a) { return a * b; }
inline H3 operator/(const H3 &a, double b) { return a * (1.0 / b); }
inline H3 operator/(double b, const H3 &a) { return recip(a) * b; }
inline H3 sqrt(const H3 &a) { const double s = ::sqrt(a.v); return chain(a, s, 0.5 / s, -0.25 / (s * a.v)); }
inline H3 log(const H3 &a) { return chain(a, ::log(a.v), 1.0 / a.v, -1.0 / (a.v * a.v)); }

}  // namespace oracle
