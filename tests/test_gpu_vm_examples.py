"""The reference's own example models on the GPU interpreter kernel.

The stored programs of ``tests/golden/vm_examples.npz`` (see
``test_vm_examples_cpu``) run through the C-ABI, bit-exact against the
checksums of the reference's own generated kernels, as stored and
optimised."""
import binascii
import ctypes

import numpy as np
import pytest

from xentica_gb300 import _native as nat
from tests.test_vm_examples_cpu import _cases, load_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("optimised", [False, True])
@pytest.mark.parametrize("name", _cases())
def test_reference_example_on_the_interpreter(name, optimised):
    """As stored, and after the compiler's straight-line optimisation (the
    form models compile to)."""
    desc, programs, c = load_case(name)
    if optimised:
        from xentica_gb300.core import vm
        programs = [vm.optimize(code, consts) for code, consts, _ in programs]
    lib = nat.load()
    h = ctypes.c_void_p()
    nat.check(lib.xk_model_create(ctypes.byref(desc), ctypes.byref(h)), "xk_model_create")
    try:
        for which, (code, consts, nregs) in enumerate(programs):
            nat.check(lib.xk_vm_load(h, which, nat.ptr(code), len(code), nat.ptr(consts),
                                     len(consts), nregs), "xk_vm_load")
        params = np.ascontiguousarray(c["params"], dtype=np.uint64)
        if params.size:
            nat.check(lib.xk_vm_set_params(h, nat.ptr(params), params.size), "xk_vm_set_params")
        init = np.ascontiguousarray(c["init"])
        n = init.size
        nat.check(lib.xk_upload(h, nat.ptr(init), n), "xk_upload")
        col0 = np.ascontiguousarray(c["init_col"], dtype=np.int32)
        nat.check(lib.xk_upload_colors(h, nat.ptr(col0), n), "xk_upload_colors")
        nat.check(lib.xk_step(h, int(c["steps"])), "xk_step")
        cells = np.empty_like(init)
        nat.check(lib.xk_download(h, nat.ptr(cells), n), "xk_download")
        col = np.empty(3 * n, dtype=np.int32)
        nat.check(lib.xk_download_colors(h, nat.ptr(col), n), "xk_download_colors")
    finally:
        lib.xk_model_destroy(h)
    assert binascii.crc32(cells.tobytes()) == int(c["cells_crc"]), name
    assert binascii.crc32(col.tobytes()) == int(c["colors_crc"]), name
