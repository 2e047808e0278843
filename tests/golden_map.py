"""Map the reference's named FacWaveformCoeffs fields (include/EOB.hh:17-362)
onto the dense per-(l, m) layout of eobgpu_gb300/csrc/physics/fac_coeffs.h."""
import re

NUMLM = 35
RHODEG = 12


def lm_index(l, m):
    return (l - 2) * (l + 1) // 2 + (m - 1)


def dense_offsets():
    """Offsets (in doubles) of the arrays of struct FacCoeffs."""
    off = {}
    o = 0
    off["rho"] = o; o += NUMLM * (RHODEG + 1)
    off["rhol"] = o; o += NUMLM * (RHODEG + 1)
    off["fre"] = o; o += NUMLM * 8
    off["fim_vh6"] = o; o += NUMLM
    off["dvh"] = o; o += NUMLM * 10
    off["dv"] = o; o += NUMLM * 9
    return off


_PAT = re.compile(r"^(delta|rho|f)(\d)(\d)(vh|v)(\d*)(l|c|S|lS)?$")


def dense_index(name):
    """Dense offset of a reference field, or None for fields with no role
    in the waveform (the *S spin variants are never read by the reference)."""
    mt = _PAT.match(name)
    if not mt:
        return None
    kind, l, m, var, k, suf = mt.groups()
    l, m = int(l), int(m)
    k = int(k) if k else 1
    if suf in ("S", "lS"):
        return None
    off = dense_offsets()
    i = lm_index(l, m)
    if kind == "rho":
        base = off["rhol"] if suf == "l" else off["rho"]
        return base + i * (RHODEG + 1) + k
    if kind == "f":
        if var == "vh":
            return off["fim_vh6"] + i
        return off["fre"] + i * 8 + k
    if kind == "delta":
        if var == "vh":
            return off["dvh"] + i * 10 + k
        return off["dv"] + i * 9 + k
    return None
