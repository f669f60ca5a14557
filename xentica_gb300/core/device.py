"""Device side of a model: the ``model.gpu`` object.

Replaces the reference's ``GPU`` / ``GPUKernels`` / ``GPUArrays``
(``xentica/core/base.py:527-589``).  ``gpu.arrays.cells.get()`` and
``gpu.arrays.colors.get()`` return the reference layout -- ``cells`` is
``cells_num * (N + 1) + 1`` packed cells with the main state in plane 0 (the
buffer planes of the reference are never materialised on the GB300 path and
read back as zeros) and ``colors`` is ``3 * cells_num`` int32.

The libxk model is created on first use (first step, render or read after a
step), so a model can be built and seeded on a machine without a GPU; any
device operation there raises :class:`XenticaException`.
"""
import numpy as np

from xentica_gb300 import _native as nat
from xentica_gb300.core.templates import match
from xentica_gb300.core.exceptions import XenticaException

__all__ = ['GPU', 'GPUArrays']


class DeviceArray:
    """Read-only view with the ``get()`` method of a PyCUDA ``GPUArray``."""

    def __init__(self, getter, shape, dtype):
        self._getter = getter
        self.shape = shape
        self.dtype = np.dtype(dtype)

    def get(self):
        """Copy to a new host array."""
        return self._getter()


class GPUArrays:
    """``cells``, ``colors`` and ``img`` of a model."""

    def __init__(self, gpu):
        self._gpu = gpu
        n = gpu.cells_num
        self.cells = DeviceArray(gpu.get_cells, (n * gpu.planes + 1, ), gpu.dtype)
        self.colors = DeviceArray(gpu.get_colors, (n * 3, ), np.int32)
        self.img = None

    def init_img(self, num_cells):
        """Allocate the viewport image (``num_cells`` int32 values)."""
        self.img = DeviceArray(lambda: np.zeros(num_cells, dtype=np.int32),
                               (num_cells, ), np.int32)


class GPU:
    """Device model behind a ``CellularAutomaton``."""

    def __init__(self, model, init_cells, init_colors):
        self.model = model
        self.template = match(model)
        self.cells_num = model.cells_num
        self.planes = len(model.buffers) + 1
        self.dtype = np.dtype(model.main.dtype)
        self._host_cells = np.ascontiguousarray(init_cells[:self.cells_num], dtype=self.dtype)
        self._host_colors = np.ascontiguousarray(init_colors, dtype=np.int32)
        self._handle = None
        self._lib = None
        self._rule = None
        self.arrays = GPUArrays(self)

    # -- device model ------------------------------------------------------
    def _ensure(self):
        if self._handle is not None:
            return
        lib = nat.load()
        desc = self.template.descriptor()
        handle = nat.ctypes.c_void_p()
        nat.check(lib.xk_model_create(nat.ctypes.byref(desc), nat.ctypes.byref(handle)),
                  "xk_model_create")
        self._lib = lib
        self._handle = handle
        if hasattr(self.template, "after_create"):
            self.template.after_create(lib, handle)
        self._rule = (desc.rule0, desc.rule1, list(desc.color_lut))
        self._upload(self._host_cells, self._host_colors)
        self._host_cells = None
        self._host_colors = None

    def _upload(self, cells, colors):
        cells = np.ascontiguousarray(cells, dtype=self.dtype)
        colors = np.ascontiguousarray(colors, dtype=np.int32)
        nat.check(self._lib.xk_upload(self._handle, nat.ptr(cells), self.cells_num), "xk_upload")
        nat.check(self._lib.xk_upload_colors(self._handle, nat.ptr(colors), self.cells_num),
                  "xk_upload_colors")
        if hasattr(self.template, "history_free") and colors.size:
            rng = (nat.ctypes.c_int32 * 2)()
            nat.check(self._lib.xk_colors_range(self._handle, rng), "xk_colors_range")
            hf = self.template.history_free(self._rule[2], (int(rng[0]), int(rng[1])))
            nat.check(self._lib.xk_set_color_mode(self._handle, int(hf)), "xk_set_color_mode")

    def __del__(self):
        if getattr(self, "_handle", None) is not None and self._lib is not None:
            try:
                self._lib.xk_model_destroy(self._handle)
            except Exception:  # interpreter shutdown
                pass
            self._handle = None

    def _bind_params(self):
        tpl = self.template
        if hasattr(tpl, "bind"):
            tpl.bind(self._lib, self._handle)
            return
        if not getattr(tpl, "param_names", None):
            return
        rule0, rule1, lut = tpl.rule_for(tpl.current_params())
        if (rule0, rule1, list(lut)) == self._rule:
            return
        old_lut = self._rule[2]
        lut_arr = (nat.ctypes.c_int32 * 6)(*lut)
        nat.check(self._lib.xk_life_set_rule(self._handle, rule0, rule1, lut_arr),
                  "xk_life_set_rule")
        if list(lut) != old_lut:
            vals = [v * (tpl._fades()[2] if tpl.color is not None else 1) for v in old_lut]
            hf = tpl.history_free(lut, (min(vals), max(vals)))
            nat.check(self._lib.xk_set_color_mode(self._handle, int(hf)), "xk_set_color_mode")
        self._rule = (rule0, rule1, list(lut))

    # -- operations used by CellularAutomaton -------------------------------
    def _plan(self):
        """Launch plan of a 2-D Life-like lattice: from the tuning cache, or
        timed and stored there (once per model)."""
        if getattr(self, "_planned", False):
            return
        self._planned = True
        topo = self.model.topology
        if topo.dimensions != 2 or not hasattr(self.template, "history_free"):
            return
        border = topo.border
        if isinstance(border, __import__("xentica_gb300.core.topology.border",
                                         fromlist=["TorusBorder"]).TorusBorder):
            kind = "torus"
        else:
            kind = "static%d" % int(getattr(border, "value", 0) or 0)
        from xentica_gb300 import tuning
        self.plan = tuning.lattice_plan(self._lib, self._handle, self.model.size[0],
                                        self.model.size[1], kind)

    def step(self, nsteps=1):
        """Advance ``nsteps`` generations with the current parameter values."""
        self._ensure()
        self._bind_params()
        self._plan()
        nat.check(self._lib.xk_step(self._handle, int(nsteps)), "xk_step")

    def render(self, width, height, zoom, dx, dy):
        """RendererPlain image as int32 ``width * height * 3``."""
        if not isinstance(self.model.renderer, __import__(
                "xentica_gb300.core.renderers", fromlist=["RendererPlain"]).RendererPlain):
            raise XenticaException("only RendererPlain is implemented on the GB300 path")
        self._ensure()
        img = np.zeros(width * height * 3, dtype=np.int32)
        nat.check(self._lib.xk_render(self._handle, nat.ptr(img), width, height, zoom, dx, dy),
                  "xk_render")
        return img

    def step_frames(self, nsteps, width, height, zoom, dx, dy, out, on_device=False):
        """Advance ``nsteps`` generations, rendering a ``width x height``
        RendererPlain frame (uint8 RGB) after each one into row ``g`` of
        ``out``: a host array of ``nsteps * width * height * 3`` bytes
        (page-locked memory lets the copies overlap the next generations), or,
        with ``on_device``, the device address of a buffer that size."""
        if not isinstance(self.model.renderer, __import__(
                "xentica_gb300.core.renderers", fromlist=["RendererPlain"]).RendererPlain):
            raise XenticaException("only RendererPlain is implemented on the GB300 path")
        self._ensure()
        self._bind_params()
        if on_device:
            addr = int(out)
        else:
            if out.dtype != np.uint8 or not out.flags.c_contiguous or \
                    out.size != int(nsteps) * width * height * 3:
                raise XenticaException("frames buffer must be contiguous uint8 of "
                                       "nsteps * width * height * 3 values")
            addr = out.ctypes.data
        nat.check(self._lib.xk_step_frames(self._handle, int(nsteps), width, height, zoom, dx, dy,
                                           nat.ctypes.c_void_p(addr), int(bool(on_device))),
                  "xk_step_frames")
        return self._lib.xk_last_step_ms()

    def mass_totals(self, count):
        """Total mass after each generation of the last ``step(count)`` (mass
        transfer models): the conserved quantity."""
        self._ensure()
        out = np.zeros(int(count), dtype=np.uint64)
        nat.check(self._lib.xk_mass_totals(self._handle, nat.ptr(out), int(count)),
                  "xk_mass_totals")
        return out

    def main_plane(self):
        """Main state in the reference dtype (``cells_num`` values)."""
        if self._handle is None:
            return self._host_cells.copy()
        out = np.empty(self.cells_num, dtype=self.dtype)
        nat.check(self._lib.xk_download(self._handle, nat.ptr(out), self.cells_num),
                  "xk_download")
        return out

    def get_cells(self):
        """Reference layout: main plane, N zeroed buffer planes, one spare."""
        out = np.zeros(self.cells_num * self.planes + 1, dtype=self.dtype)
        out[:self.cells_num] = self.main_plane()
        return out

    def get_colors(self):
        """Colours (``3 * cells_num`` int32)."""
        if self._handle is None:
            return self._host_colors.copy()
        out = np.empty(self.cells_num * 3, dtype=np.int32)
        nat.check(self._lib.xk_download_colors(self._handle, nat.ptr(out), self.cells_num),
                  "xk_download_colors")
        return out

    def load(self, cells, colors):
        """Replace state and colours (reference ``save()`` layout accepted)."""
        cells = np.asarray(cells)[:self.cells_num].astype(self.dtype, copy=False)   # no host copy when typed
        colors = np.asarray(colors, dtype=np.int32)
        if self._handle is None:
            # kept until the device model exists: copies, not views of the caller's arrays
            self._host_cells = np.array(cells, copy=True, order="C")
            self._host_colors = np.array(colors, copy=True, order="C")
            return
        self._upload(cells, colors)
