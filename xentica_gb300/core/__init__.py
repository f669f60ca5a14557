"""Core classes of the framework (reference ``xentica/core/__init__.py``).

Shortcuts: ``CellularAutomaton``, ``Experiment``, ``OrthogonalLattice``,
``MooreNeighborhood``, ``VonNeumannNeighborhood``, ``TorusBorder``,
``StaticBorder``, ``IntegerProperty``, ``FloatProperty``,
``TotalisticRuleProperty``, ``RandomProperty``, ``Parameter``,
``IntegerVariable``, ``FloatVariable``.
"""
from xentica_gb300.core.base import CellularAutomaton
from xentica_gb300.core.properties import (
    IntegerProperty,
    FloatProperty,
    TotalisticRuleProperty,
    RandomProperty,
)
from xentica_gb300.core.variables import IntegerVariable, FloatVariable
from xentica_gb300.core.parameters import Parameter
from xentica_gb300.core.topology.lattice import OrthogonalLattice
from xentica_gb300.core.topology.neighborhood import MooreNeighborhood, VonNeumannNeighborhood
from xentica_gb300.core.topology.border import TorusBorder, StaticBorder
from xentica_gb300.core.experiment import Experiment

__all__ = [
    'CellularAutomaton', 'IntegerProperty', 'FloatProperty',
    'TotalisticRuleProperty', 'RandomProperty', 'Parameter',
    'IntegerVariable', 'FloatVariable', 'OrthogonalLattice',
    'MooreNeighborhood', 'VonNeumannNeighborhood', 'TorusBorder',
    'StaticBorder', 'Experiment',
]
