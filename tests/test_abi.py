"""The C-ABI library loads on a machine without a GPU and exports every
function that include/*.h declares (no compute calls)."""
import os
import re

from qll_gb300 import qll

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for fn in sorted(os.listdir(INC)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(INC, fn)).read()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
        text = re.sub(r"//[^\n]*", " ", text)
        text = re.sub(r"#[^\n]*", " ", text)
        text = re.sub(r"\{[^{}]*\}", " ", text)
        text = re.sub(r"typedef[^;]*;", " ", text)
        for m in re.finditer(r"(PR\((\w+)\)|\b(\w+))\s*\([^;()]*(\([^;()]*\)[^;()]*)*\)\s*;",
                             text):
            if m.group(2):
                names.add(m.group(2) + "D")
                names.add(m.group(2) + "F")
            elif m.group(3) not in ("if", "while", "for", "return", "sizeof"):
                names.add(m.group(3))
    return names


def test_headers_declare_the_hot_path():
    names = declared_functions()
    for must in ("dslash2D", "solve2F", "solveMulti2D", "createStaggeredSolverD", "cgSolveD",
                 "smearFat7D", "wilsonDslashF", "layoutIndex", "qllg_stag_solve",
                 "qllg_gen_gauge"):
        assert must in names, must


def test_library_exports_every_declared_symbol():
    L = qll.load()
    missing = [n for n in sorted(declared_functions()) if not hasattr(L, n)]
    assert not missing, missing


def test_library_loads_without_gpu_and_reports_errors():
    L = qll.load()
    assert b"sm_103a" in L.qllg_version()
    # geometry validation is host logic: odd extents are refused with a message
    import ctypes
    V = 3*4*4*4
    out = (ctypes.c_int*V)()
    rc = L.qllg_stag_nbr_table(qll.dims_c((3, 4, 4, 4)), 0, 0, out)
    assert rc < 0
    assert qll.last_error()


def test_documented_parameters_exist_with_their_defaults():
    """every solver parameter the header documents is known to the library,
    with the default the header states (no GPU needed: the table is host
    state)"""
    import ctypes
    text = open(os.path.join(INC, "qll_gb300.h")).read()
    block = text[text.index("/* solver parameters (name, default):"):]
    block = block[:block.index("*/")]
    documented = re.findall(r'"(\w+)" \(([-0-9.e]+)', block)
    assert len(documented) >= 15
    L = qll.load()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    L.qllg_set_param.restype = ctypes.c_int
    L.qllg_get_param.argtypes = [ctypes.c_char_p]
    L.qllg_get_param.restype = ctypes.c_double
    for name, default in documented:
        assert L.qllg_get_param(name.encode()) == float(default), name
        assert L.qllg_set_param(name.encode(), float(default)) == 0, name
    assert L.qllg_set_param(b"no_such_parameter", 1.0) == -1
    # and the header documents every parameter of the library's table
    table = re.findall(r'\{"(\w+)",', open(os.path.join(ROOT, "qll_gb300", "csrc", "runtime.c")).read())
    assert set(table) == {n for n, _ in documented}
