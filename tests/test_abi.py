"""The C-ABI library: it builds, loads without a GPU, exports every symbol
``include/xk.h`` declares, and the ctypes descriptor matches the C layout."""
import ctypes
import os
import re
import subprocess

import pytest

from xentica_gb300 import _native as nat
from xentica_gb300 import build as xk_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xk.h")


@pytest.fixture(scope="module")
def lib():
    xk_build.build()
    return nat.load()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xk_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_functions():
    names = declared_functions()
    assert "xk_model_create" in names and "xk_batch_step" in names and len(names) >= 20


def test_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in nat.SIGNATURES, "no ctypes signature for %s" % name


def test_last_error_without_gpu(lib):
    # a null-argument call fails with a status and a message, never aborts
    assert lib.xk_model_create(None, None) == -1
    assert "null" in nat.last_error()


def test_desc_layout_matches_c(tmp_path):
    fields = [f[0] for f in nat.XkDesc._fields_]
    src = tmp_path / "layout.c"
    body = "".join('printf("%%s %%zu\\n", "%s", offsetof(xk_desc, %s));\n' % (f, f) for f in fields)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "%s"\nint main(void){\n'
                   'printf("__sizeof__ %%zu\\n", sizeof(xk_desc));\n%s return 0; }\n' % (HEADER, body))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(line.split() for line in out if line)
    assert int(got["__sizeof__"]) == ctypes.sizeof(nat.XkDesc)
    for f in fields:
        assert int(got[f]) == getattr(nat.XkDesc, f).offset, f


@pytest.mark.parametrize("family,field,value", [
    (nat.XK_FAMILY_GRAVITY, "state_bytes", 4),
    (nat.XK_FAMILY_GRAVITY, "nbr", 4),
    (nat.XK_FAMILY_GRAVITY, "color_kind", nat.XK_COLOR_PLAIN),
    (nat.XK_FAMILY_LIFECOLOR, "state_bytes", 8),
    (nat.XK_FAMILY_LIFECOLOR, "ndim", 3),
    (nat.XK_FAMILY_NOISE, "state_bytes", 4),
    (nat.XK_FAMILY_EVOLIFE, "torus", 0),
    (99, "family", 99),
])
def test_fused_families_reject_other_descriptors(lib, family, field, value):
    """A descriptor a fused family's kernel cannot run is refused with a
    status (before any device work, so this runs without a GPU)."""
    from tests.models import GraviCowboys, GraviExperiment
    d = GraviCowboys(GraviExperiment).gpu.template.descriptor()
    d.family = family
    if family == nat.XK_FAMILY_LIFECOLOR:
        d.state_bytes = 4
    elif family == nat.XK_FAMILY_NOISE:
        d.state_bytes = 2
    setattr(d, field, value)
    h = ctypes.c_void_p()
    rc = lib.xk_model_create(ctypes.byref(d), ctypes.byref(h))
    assert rc in (nat.XK_ERR_ARG, nat.XK_ERR_UNSUPPORTED), rc
    assert not h.value
    assert nat.last_error()
