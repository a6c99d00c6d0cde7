"""qll_gb300 -- GB300-native (sm_103a) rebuild of the QLL lattice-QCD solver
hot path: asqtad staggered and Wilson Dslash, CG and multishift CG, fat7
smearing.  The product is the C library libqll_gb300.so (QLL's C API plus a
native qllg_* API, headers in include/); this package holds its sources
(csrc/), its build step (build.py) and ctypes bindings (qll.py)."""
from . import qll  # noqa: F401
from .qll import load, last_error  # noqa: F401
