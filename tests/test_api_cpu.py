"""The reference's host-side tests, run against xentica_gb300 (no GPU needed).

Ports of ``tests/core/test_variables.py``, ``test_properties.py`` (non-kernel
parts), ``topology/*``, ``test_mixins.py``, ``test_renderers.py``,
``tests/seeds/*``, ``tests/tools/*``, ``tests/utils/*`` and
``tests/bridge/test_base.py`` of the reference.  Models are built and seeded
on the host; nothing here touches a device.
"""
import binascii

import numpy as np
import pytest

from xentica_gb300 import core, seeds
from xentica_gb300.core import color_effects
from xentica_gb300.bridge.base import Bridge
from xentica_gb300.core.base import CellularAutomaton
from xentica_gb300.core.exceptions import XenticaException
from xentica_gb300.core.mixins import BscaDetectorMixin
from xentica_gb300.core.properties import (
    Property, IntegerProperty, ContainerProperty, TotalisticRuleProperty)
from xentica_gb300.core.renderers import Renderer, RendererPlain
from xentica_gb300.core.topology.border import TorusBorder
from xentica_gb300.core.topology.lattice import OrthogonalLattice
from xentica_gb300.core.topology.neighborhood import MooreNeighborhood
from xentica_gb300.core.variables import Variable, IntegerVariable
from xentica_gb300.seeds.patterns import ValDict, BigBang, PrimordialSoup
from xentica_gb300.seeds.random import RandInt, LocalRandom, RandBernoulli, RandPoisson
from xentica_gb300.tools import xmath
from xentica_gb300.tools.rules import LifeLike
from xentica_gb300.utils.formatters import sizeof_fmt

from tests.models import GameOfLife, GOLExperiment


# -- variables (reference tests/core/test_variables.py) ----------------------

class InvertCA(core.CellularAutomaton):
    """Inverts each cell every step."""
    state = core.IntegerProperty(max_val=1)
    intvar = IntegerVariable()

    class Topology:
        dimensions = 2
        lattice = core.OrthogonalLattice()
        neighborhood = core.MooreNeighborhood()
        border = core.TorusBorder()

    def emit(self):
        self.intvar = self.main.state
        self.buffers[0].state = self.intvar

    def absorb(self):
        self.intvar = self.buffers[0].state
        self.main.state = -self.intvar
        var_list = [IntegerVariable(name="self_var"), IntegerVariable()]
        var_list[1] += 1

    def color(self):
        """No colour."""


class InvertExperiment(core.Experiment):
    word = "INSIDE OUT"
    size = (64, 36, )
    seed = seeds.patterns.PrimordialSoup(vals={"state": seeds.random.RandInt(0, 1)})


def test_variable_names():
    myvar1 = IntegerVariable()
    assert str(myvar1) == "myvar1"
    assert myvar1.code == "myvar1"
    myvar2 = IntegerVariable(1)
    assert str(myvar2) == "myvar2"
    var_list = [IntegerVariable(1, name="myvar3"), IntegerVariable(name="myvar4"),
                IntegerVariable(2), IntegerVariable()]
    assert var_list[0].var_name == "myvar3"
    assert var_list[1].var_name == "myvar4"
    assert var_list[2].var_name == "var"
    assert var_list[3].var_name == "var"


def test_variable_descriptor_listing():
    # exact traced listing the reference asserts for its generated C
    # (reference tests/core/test_variables.py:109-144); InvertCA has no
    # GB300 template, so only the translator is exercised
    model = InvertCA.__new__(InvertCA)
    Translator_init(model)
    correct_emit = """
unsigned char _cell_state;
int tmp__cell;
tmp__cell = (_cell) & 1;
_cell_state = tmp__cell;
unsigned int intvar = 0;
intvar = _cell_state;
unsigned char _bcell_state0;
_bcell_state0 = intvar;
unsigned char _bcell0;
_bcell0 = ((unsigned char) _bcell_state0 & 1);
fld[i + n * 8] = _bcell0;
"""
    correct_absorb = """
unsigned char _bcell_state0;
int tmp__bcell0;
tmp__bcell0 = (_bcell0) & 1;
_bcell_state0 = tmp__bcell0;
unsigned int intvar = 0;
intvar = _bcell_state0;
unsigned char _cell_state;
_cell_state = (-(intvar));
unsigned char _cell = fld[i];
unsigned int var = 0;
var += 1;
_cell = ((unsigned char) _cell_state & 1);
fld[i] = _cell;
"""
    assert correct_emit in model.cuda_source
    assert correct_absorb in model.cuda_source


def Translator_init(model):
    """Run only the tracing half of ``CellularAutomaton.__init__``."""
    from xentica_gb300.core.base import Translator
    Translator.__init__(model)
    for name in ("word", "size"):
        setattr(model, name, getattr(InvertExperiment, name))
    model.cells_num = int(np.prod(model.size))
    model.build_source()


def test_illegal_assign():
    class BrokenCA(InvertCA):
        def emit(self):
            deferred_exp = 1 + self.main.state
            deferred_exp += 1
    with pytest.raises(XenticaException):
        BrokenCA(InvertExperiment)


def test_no_init_val():
    with pytest.raises(XenticaException):
        Variable()


class RawColorEffect(color_effects.ColorEffect):
    """A colour effect with its own C text, which no GB300 kernel runs."""

    def __call__(self):
        self.effect = "new_r = new_r ^ 7;"
        return super().__call__()


class RawColorLife(GameOfLife):
    @RawColorEffect
    def color(self):
        return (self.main.state * 255, 0, 0)


def test_no_template_raises():
    # a model no family implements and the interpreter cannot run (C text
    # of its own) fails loudly at construction
    with pytest.raises(XenticaException, match="No GB300 kernel template"):
        RawColorLife(GOLExperiment)


def test_interpreter_takes_other_models():
    # inverting models are not a hand-written family: the interpreter runs them
    model = InvertCA(InvertExperiment)
    assert type(model.gpu.template).__name__ == "VMTemplate"


# -- properties (reference tests/core/test_properties.py) -------------------

def test_property_widths():
    assert IntegerProperty(max_val=1).width == 1
    assert Property().bit_width == 1
    prop = IntegerProperty(max_val=10e23)
    assert prop.bit_width == 80
    assert prop.width == 2


def test_property_set_descriptor():
    prop = Property()
    prop.cont = ContainerProperty()
    prop.cont.var_name = "foo"
    prop.cont = 1
    assert type(prop.cont).__name__ == "ContainerProperty"


def test_unbound_property():
    prop = Property()
    with pytest.raises(XenticaException):
        assert not prop.declared
    with pytest.raises(XenticaException):
        assert prop.coords_declared
    with pytest.raises(XenticaException):
        assert not ContainerProperty().unpacked


def test_container_values():
    assert len(list(GameOfLife.main.values())) == 1


def test_pure_totalistic():
    prop = TotalisticRuleProperty(outer=False)
    with pytest.raises(XenticaException):
        prop.is_sustained(8)
    with pytest.raises(XenticaException):
        prop.is_born(8)
    prop.var_name = "rule"
    assert str(prop.next_val(1, 3)) == "((rule >> 4) & 1)"


def test_outer_totalistic_text():
    class GolTest(GameOfLife):
        rule = TotalisticRuleProperty(outer=True)

        def absorb(self):
            GameOfLife.absorb(self)
    from xentica_gb300.core.base import Translator
    model = GolTest.__new__(GolTest)
    Translator.__init__(model)
    model.size = (8, 8)
    assert str(model.main.rule.is_sustained(8)) == "(((_cell_rule & 261120) >> 17) & 1)"
    assert str(model.main.rule.is_born(8)) == "(((_cell_rule & 510) >> 8) & 1)"
    assert str(model.main.rule.next_val(1, 3)) == "((_cell_rule >> 12) & 1)"


# -- topology, mixins, renderers ----------------------------------------------

def test_topology_dimensions():
    for obj in (TorusBorder(), OrthogonalLattice(), MooreNeighborhood()):
        with pytest.raises(XenticaException):
            obj.dimensions = 0


def test_wrong_field_size():
    class Broken(GOLExperiment):
        size = (23, )
    with pytest.raises(XenticaException):
        GameOfLife(Broken)


def test_no_topology():
    with pytest.raises(XenticaException):
        class NoTopologyCA(CellularAutomaton):
            pass
    with pytest.raises(XenticaException):
        class NoLatticeCA(CellularAutomaton):
            class Topology:
                pass


def test_bsca_not_detected():
    class Dummy(BscaDetectorMixin):
        @property
        def test_bsca(self):
            return self.bsca
    with pytest.raises(XenticaException):
        Dummy().test_bsca


def test_renderers():
    assert Renderer().render_code() == ""
    assert RendererPlain(projection_axes=(1, 0)).projection_axes == (1, 0)


def test_unset_viewport():
    model = GameOfLife(GOLExperiment)
    with pytest.raises(XenticaException):
        model.render()


# -- seeds (reference tests/seeds/*) ------------------------------------------

def test_valdict():
    assert ValDict({'s': 3})['s'] == 3
    vd = ValDict({'a': 2, 's': RandInt(11, 23), 'd': 3.3})
    for _ in range(10):
        assert 11 <= vd['s'] <= 23
    assert vd['d'] == 3.3
    with pytest.raises(KeyError):
        vd['x']
    with pytest.raises(NotImplementedError):
        vd['a'] = 2
    for key, val in vd.items():
        if key == 'a':
            assert val == 2


def test_random_known_answers():
    rng = LocalRandom("test")
    assert [rng.standard.randint(11, 23) for _ in range(10)] == [22, 15, 21, 23, 14, 14, 11, 20, 17, 23]
    rng = LocalRandom("test")
    assert list(rng.numpy.randint(11, 23, (10, ))) == [19, 16, 22, 19, 15, 22, 20, 20, 13, 15]

    class Holder:
        def __init__(self, seed=None):
            self.random = LocalRandom(seed)
    holder = Holder("test")
    Holder.rand_val = RandInt(11, 23)
    assert [holder.rand_val for _ in range(10)] == [22, 15, 21, 23, 14, 14, 11, 20, 17, 23]


def test_primordial_soup_checksum():
    # a fresh seed pattern: patterns clamp their area to the field in place,
    # so resizing an experiment that shares one would change it for others
    bsca = GameOfLife(type("E", (GOLExperiment, ), {"size": (100, 100), "seed": PrimordialSoup(
        vals={'state': RandInt(0, 1)})}))
    seed = PrimordialSoup(vals={'state': RandInt(0, 1)})
    cells = np.zeros((10000, ), dtype=np.int32)
    seed.random = LocalRandom("test")
    seed.generate(cells, bsca)
    assert binascii.crc32(cells[:10000]) == 1648433356


def test_big_bang_area():
    exp = type("E", (GOLExperiment, ), {"size": (100, 100), "seed": BigBang(
        pos=(32, 20), size=(10, 10), vals={"state": RandInt(0, 1)})})
    bsca = GameOfLife(exp)
    cells = bsca.gpu.arrays.cells.get()[:bsca.cells_num]
    for i in np.where(cells == 1)[0]:
        x, y = i % 100, i // 100
        assert 32 <= x <= 42 and 20 <= y <= 30
    for kwargs in ({"pos": (10, 10)}, {"size": (10, 10)}, {}):
        pattern = BigBang(vals={'state': RandInt(0, 1)}, **kwargs)
        cells = np.zeros((10000, ), dtype=np.int32)
        pattern.generate(cells, bsca)
        assert np.sum(cells) > 0
    pattern = BigBang(pos=(90, 90), size=(20, 20), vals={'state': RandInt(0, 1)})
    pattern.generate(np.zeros((10000, ), dtype=np.int32), bsca)
    assert tuple(pattern.pos) == (80, 80)


def test_bernoulli_poisson_seeds():
    class Holder:
        size = (50, 40)

        def __init__(self):
            self.random = LocalRandom("bp")
    h = Holder()
    b = RandBernoulli(0.3).__get__(h, Holder)
    assert b.shape == (2000, ) and set(np.unique(b)) <= {0, 1}
    ref = (LocalRandom("bp").numpy.random_sample(2000) < 0.3).astype(np.int64)
    assert np.array_equal(b, ref)
    p = RandPoisson(4).__get__(Holder(), Holder)
    assert np.array_equal(p, LocalRandom("bp").numpy.poisson(4, 2000))


# -- tools, utils -------------------------------------------------------------

def test_golly():
    assert LifeLike.golly2int("B3/S23") == 6152
    assert LifeLike.int2golly(6152) == "B3/S23"


def test_xmath_text():
    assert str(xmath.popc("x")) == "(__popc(x))"
    assert str(xmath.exp("x")) == "(exp(x))"
    assert str(xmath.min(1, "a", "b")) == \
        "(((((1) < (a)) ? (1) : (a)) < (b)) ? (((1) < (a)) ? (1) : (a)) : (b))"


def test_sizeof_fmt():
    assert sizeof_fmt(345) == "345"
    assert sizeof_fmt(34567) == "34.57K"
    assert sizeof_fmt(34567 * (10 ** 12)) == "34.57P"
    assert sizeof_fmt(34567 * (10 ** 21)) == "34.57Y"


# -- bridge (reference tests/bridge/test_base.py) ----------------------------

class SysInfo:
    def toggle(self):
        self.toggled = True


class DummyGui:
    def __init__(self):
        self.sysinfo = SysInfo()

    def exit_app(self):
        self.exited = True


def test_bridge_actions():
    model = GameOfLife(type("E", (GOLExperiment, ), {"pos": [0, 0]}))
    gui = DummyGui()
    Bridge.noop(model, gui)
    Bridge.exit_app(model, gui)
    assert gui.exited
    y = model.pos[1]
    model.bridge.key_actions['up'](model, gui)
    assert model.pos[1] == (y + 1) % model.size[1]
    model.bridge.key_actions['down'](model, gui)
    assert model.pos[1] == y
    x = model.pos[0]
    model.bridge.key_actions['right'](model, gui)
    assert model.pos[0] == (x + 1) % model.size[0]
    model.bridge.key_actions['left'](model, gui)
    assert model.pos[0] == x
    zoom = model.zoom
    model.bridge.key_actions['='](model, gui)
    assert model.zoom == zoom + 1
    model.bridge.key_actions['-'](model, gui)
    model.bridge.key_actions['-'](model, gui)
    assert model.zoom == max(zoom - 1, 1)
    speed = model.speed
    model.bridge.key_actions[']'](model, gui)
    assert model.speed == speed + 1
    model.bridge.key_actions['['](model, gui)
    model.bridge.key_actions['['](model, gui)
    assert model.speed == max(speed - 1, 1)
    paused = model.paused
    Bridge.toggle_pause(model, gui)
    assert model.paused != paused
    Bridge.toggle_sysinfo(model, gui)
    assert gui.sysinfo.toggled


def test_template_match_repeated_instances():
    # the translator's container state carries over between models of one
    # class (a buffer read by one kernel is declared with a load in the next
    # model's kernels); every instance must still match its kernel family
    from xentica_gb300.core import canonical
    from tests.models import MassTransfer, MassExperiment, EvoLife, BigBangExperiment
    small = type("E", (MassExperiment, ), {"size": (12, 10, 8)})
    for cls in (MassTransfer, canonical.MassTransferProgram, MassTransfer):
        for _ in range(2):
            assert type(cls(small).gpu.template).__name__ == "MassTemplate"
    evo = type("E", (BigBangExperiment, ), {"size": (128, 128)})
    for _ in range(2):
        assert type(EvoLife(evo).gpu.template).__name__ == "EvoLifeTemplate"


def test_headless_viewer_keys_and_ppm(tmp_path):
    from xentica_gb300.bridge.headless import HeadlessViewer, write_ppm
    model = GameOfLife(type("E", (GOLExperiment, ), {"pos": [0, 0]}))
    viewer = HeadlessViewer(model, (64, 36))
    zoom, pos = model.zoom, list(model.pos)
    for key in ("]", "]", "=", "right", "up", "spacebar", "f12", "unbound-key"):
        viewer.press(key)
    assert model.speed == 3 and model.zoom == zoom + 1 and model.paused
    assert model.pos == [(pos[0] + 1) % model.size[0], (pos[1] + 1) % model.size[1]]
    assert viewer.sysinfo.shown and viewer.running
    viewer.press("escape")
    assert not viewer.running
    assert viewer.run(5) == 0                    # exited: no frame drawn
    img = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3)
    write_ppm(str(tmp_path / "f.ppm"), img)
    raw = open(str(tmp_path / "f.ppm"), "rb").read()
    assert raw == b"P6\n3 2\n255\n" + img.tobytes()


def test_interpreter_bytecode_reproduces_fixtures(golden):
    # the compiler's bytecode, run by the NumPy executor (the GPU kernel's
    # semantics), against the reference's checksums on small fixtures
    from tests import vm_cpu
    from tests.models import build_from_job
    from tests.test_oracle import crc
    for case in ("gol_33x9", "static_31x5", "gol_color_fade", "gol_plain_color", "rule_highlife",
                 "mass_24x20x12", "evolife_bigbang_mut_131x101"):
        entry = golden[case]
        model = build_from_job(entry["job"])
        n = model.cells_num
        fld = np.zeros(n * (len(model.buffers) + 1) + 1, dtype=model.main.dtype)
        fld[:n] = model.gpu.arrays.cells.get()[:n]
        col = np.zeros(3 * n, dtype=np.int32)
        cp = min(int(c) for c in entry["steps"])
        vm_cpu.step(model, fld, col, cp)
        assert crc(fld[:n]) == entry["steps"][str(cp)]["cells"], case
        assert crc(col) == entry["steps"][str(cp)]["colors"], case
