"""Initial-state (seed) generation (reference ``xentica/seeds``)."""
from xentica_gb300.seeds import random
from xentica_gb300.seeds import patterns

__all__ = ['random', 'patterns', ]
