// Second-order forward-mode dual numbers in two variables (r, pphi), used by
// the physical initial-condition option for d2H/dr2 and d2H/dr dpphi.
#pragma once
#include <math.h>
#include "fac_coeffs.h"

namespace eob {
namespace hd {

// kept in its own namespace so that argument-dependent lookup picks these
// math overloads for HD2 while plain doubles keep the global ones
struct HD2 {
    double v, g0, g1, h00, h01, h11;
    EOB_HD HD2() : v(0), g0(0), g1(0), h00(0), h01(0), h11(0) {}
    EOB_HD HD2(double x) : v(x), g0(0), g1(0), h00(0), h01(0), h11(0) {}
};
EOB_HD HD2 hd_chain(const HD2 &a, double f0, double f1, double f2)
{
    HD2 r;
    r.v = f0;
    r.g0 = f1 * a.g0;
    r.g1 = f1 * a.g1;
    r.h00 = f1 * a.h00 + f2 * a.g0 * a.g0;
    r.h01 = f1 * a.h01 + f2 * a.g0 * a.g1;
    r.h11 = f1 * a.h11 + f2 * a.g1 * a.g1;
    return r;
}
EOB_HD HD2 operator+(const HD2 &a, const HD2 &b)
{
    HD2 r;
    r.v = a.v + b.v; r.g0 = a.g0 + b.g0; r.g1 = a.g1 + b.g1;
    r.h00 = a.h00 + b.h00; r.h01 = a.h01 + b.h01; r.h11 = a.h11 + b.h11;
    return r;
}
EOB_HD HD2 operator-(const HD2 &a) { return hd_chain(a, -a.v, -1.0, 0.0); }
EOB_HD HD2 operator-(const HD2 &a, const HD2 &b) { return a + (-b); }
EOB_HD HD2 operator*(const HD2 &a, const HD2 &b)
{
    HD2 r;
    r.v = a.v * b.v;
    r.g0 = a.v * b.g0 + b.v * a.g0;
    r.g1 = a.v * b.g1 + b.v * a.g1;
    r.h00 = a.v * b.h00 + b.v * a.h00 + 2.0 * a.g0 * b.g0;
    r.h01 = a.v * b.h01 + b.v * a.h01 + a.g0 * b.g1 + a.g1 * b.g0;
    r.h11 = a.v * b.h11 + b.v * a.h11 + 2.0 * a.g1 * b.g1;
    return r;
}
EOB_HD HD2 hd_recip(const HD2 &a) { const double iv = 1.0 / a.v; return hd_chain(a, iv, -iv * iv, 2.0 * iv * iv * iv); }
EOB_HD HD2 operator/(const HD2 &a, const HD2 &b) { return a * hd_recip(b); }
EOB_HD HD2 operator+(const HD2 &a, double b) { HD2 r = a; r.v += b; return r; }
EOB_HD HD2 operator+(double b, const HD2 &a) { return a + b; }
EOB_HD HD2 operator-(const HD2 &a, double b) { HD2 r = a; r.v -= b; return r; }
EOB_HD HD2 operator-(double b, const HD2 &a) { return HD2(b) - a; }
EOB_HD HD2 operator*(const HD2 &a, double b) { return hd_chain(a, a.v * b, b, 0.0); }
EOB_HD HD2 operator*(double b, const HD2 &a) { return a * b; }
EOB_HD HD2 operator/(const HD2 &a, double b) { return a * (1.0 / b); }
EOB_HD HD2 operator/(double b, const HD2 &a) { return hd_recip(a) * b; }
EOB_HD HD2 sqrt(const HD2 &a) { const double s = ::sqrt(a.v); return hd_chain(a, s, 0.5 / s, -0.25 / (s * a.v)); }
EOB_HD HD2 log(const HD2 &a) { return hd_chain(a, ::log(a.v), 1.0 / a.v, -1.0 / (a.v * a.v)); }

// three variables (r, pr, pphi), full symmetric Hessian
struct HD3 {
    double v, g[3], h[6];  // h: 00, 01, 02, 11, 12, 22
    EOB_HD HD3() : v(0), g{0, 0, 0}, h{0, 0, 0, 0, 0, 0} {}
    EOB_HD HD3(double x) : v(x), g{0, 0, 0}, h{0, 0, 0, 0, 0, 0} {}
};
EOB_HD HD3 hd_chain(const HD3 &a, double f0, double f1, double f2)
{
    HD3 r;
    r.v = f0;
    for (int i = 0; i < 3; ++i) r.g[i] = f1 * a.g[i];
    int q = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j, ++q) r.h[q] = f1 * a.h[q] + f2 * a.g[i] * a.g[j];
    return r;
}
EOB_HD HD3 operator+(const HD3 &a, const HD3 &b)
{
    HD3 r;
    r.v = a.v + b.v;
    for (int i = 0; i < 3; ++i) r.g[i] = a.g[i] + b.g[i];
    for (int q = 0; q < 6; ++q) r.h[q] = a.h[q] + b.h[q];
    return r;
}
EOB_HD HD3 operator-(const HD3 &a) { return hd_chain(a, -a.v, -1.0, 0.0); }
EOB_HD HD3 operator-(const HD3 &a, const HD3 &b) { return a + (-b); }
EOB_HD HD3 operator*(const HD3 &a, const HD3 &b)
{
    HD3 r;
    r.v = a.v * b.v;
    for (int i = 0; i < 3; ++i) r.g[i] = a.v * b.g[i] + b.v * a.g[i];
    int q = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j, ++q) r.h[q] = a.v * b.h[q] + b.v * a.h[q] + a.g[i] * b.g[j] + a.g[j] * b.g[i];
    return r;
}
EOB_HD HD3 hd_recip(const HD3 &a) { const double iv = 1.0 / a.v; return hd_chain(a, iv, -iv * iv, 2.0 * iv * iv * iv); }
EOB_HD HD3 operator/(const HD3 &a, const HD3 &b) { return a * hd_recip(b); }
EOB_HD HD3 operator+(const HD3 &a, double b) { HD3 r = a; r.v += b; return r; }
EOB_HD HD3 operator+(double b, const HD3 &a) { return a + b; }
EOB_HD HD3 operator-(const HD3 &a, double b) { HD3 r = a; r.v -= b; return r; }
EOB_HD HD3 operator-(double b, const HD3 &a) { return HD3(b) - a; }
EOB_HD HD3 operator*(const HD3 &a, double b) { return hd_chain(a, a.v * b, b, 0.0); }
EOB_HD HD3 operator*(double b, const HD3 &a) { return a * b; }
EOB_HD HD3 operator/(const HD3 &a, double b) { return a * (1.0 / b); }
EOB_HD HD3 operator/(double b, const HD3 &a) { return hd_recip(a) * b; }
EOB_HD HD3 sqrt(const HD3 &a) { const double s = ::sqrt(a.v); return hd_chain(a, s, 0.5 / s, -0.25 / (s * a.v)); }
EOB_HD HD3 log(const HD3 &a) { return hd_chain(a, ::log(a.v), 1.0 / a.v, -1.0 / (a.v * a.v)); }

}  // namespace hd
}  // namespace eob
