"""The C-ABI library: it builds, loads, exports every declared symbol, and
rejects bad arguments before touching the device.  No compute calls."""
import ctypes
import os
import re

import pytest

from gigalens_gb300 import _native as N
from gigalens_gb300.cuda._plan import ModelLayout
from tests.helpers import default_physmodel

HEADER_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_functions():
    names = []
    for f in sorted(os.listdir(HEADER_DIR)):
        if f.endswith(".h"):
            text = open(os.path.join(HEADER_DIR, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(gl_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    names = declared_functions()
    assert "gl_forward_grad" in names and "gl_plan_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes binding covers them all
    bound = {s[0] for s in N.SIGNATURES}
    assert set(names) <= bound, set(names) - bound


def test_abi_version():
    import re

    with open(os.path.join(HEADER_DIR, "gigalens_cuda.h")) as fh:
        hv = int(re.search(r"#define GL_ABI_VERSION (\d+)", fh.read()).group(1))
    assert N.lib().gl_abi_version() == hv == N.GL_ABI_VERSION


def test_struct_mirrors_match_the_header():
    """The ctypes mirrors have the C structs' sizes (a field added on one side
    only would shift every later field)."""
    mirrors = [N.gl_profile_desc, N.gl_model_desc, N.gl_image_desc, N.gl_prior_leaf, N.gl_tune_result,
               N.gl_adam_cfg, N.gl_tuning]
    lib = N.lib()
    for i, m in enumerate(mirrors):
        assert lib.gl_struct_size(i) == ctypes.sizeof(m), (m.__name__, lib.gl_struct_size(i), ctypes.sizeof(m))
    assert lib.gl_struct_size(len(mirrors)) == -1


def test_bad_arguments_are_rejected_without_a_device():
    lib = N.lib()
    h = ctypes.c_void_p()
    rc = lib.gl_plan_create(None, None, 0, ctypes.byref(h))
    assert rc == N.GL_ERR_INVALID and b"bad arguments" in lib.gl_last_error()
    assert lib.gl_profile_eval(N.GL_PROF_EPL, None, None, -1, None, None, None, None, None) == N.GL_ERR_INVALID
    assert lib.gl_epl_term_count(None, None, 0, 50, None, None) == N.GL_ERR_INVALID
    assert lib.gl_adam_step(None, None, None, None, 10, 1.0, None, None, None) == N.GL_ERR_INVALID
    assert lib.gl_forward(None, None, None, 4, None, None, None, None, None) == N.GL_ERR_INVALID
    assert lib.gl_plan_destroy(None) == N.GL_OK


def test_model_layout_matches_reference_packing():
    lay = ModelLayout(default_physmodel())
    assert lay.d == 22
    keys = [k for _, _, k in lay.entries]
    assert keys[:8] == ["center_x", "center_y", "e1", "e2", "gamma", "theta_E", "gamma1", "gamma2"]
    assert keys[8:15] == ["Ie", "R_sersic", "center_x", "center_y", "e1", "e2", "n_sersic"]
    epl = lay.desc.prof[0]
    assert epl.type == N.GL_PROF_EPL and epl.niter == 50
    # canonical EPL order theta_E, gamma, e1, e2, center_x, center_y -> flat columns
    assert list(epl.col)[:6] == [5, 4, 2, 3, 0, 1]
    src = lay.desc.prof[3]
    assert src.group == N.GL_GROUP_SOURCE and list(src.col)[:7] == [16, 21, 19, 20, 17, 18, 15]
