"""`eob` -- the import name of the reference's package (mikekatz04/EOBGPU),
served by this repository's GB300 implementation.

`import eob.seobnrv4phm`, `from eob.pyEOB import SEOBNRv5Class`, ... resolve to
the modules of eobgpu_gb300.eob, so code written against the reference runs
unchanged on top of libeobgb300.
"""
import importlib
import sys

_PKG = "eobgpu_gb300.eob"
_MODULES = ("seobnrv4phm", "new_Dormand_horiz", "pyEOB", "pydopr853", "pytdinterp")

for _m in _MODULES:
    _mod = importlib.import_module(f"{_PKG}.{_m}")
    sys.modules[f"{__name__}.{_m}"] = _mod
    globals()[_m] = _mod
