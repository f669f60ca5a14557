"""Experiments (reference ``xentica/core/experiment.py:42-49``).

An experiment is a class whose attributes configure a model run::

    class MyExperiment(core.Experiment):
        word = "My Special String"      # RNG seed string
        size = (640, 360, )             # field size
        zoom = 3                        # initial zoom
        pos = [0, 0]                    # initial view shift
        seed = seeds.patterns.PrimordialSoup(vals={"state": seeds.random.RandInt(0, 1)})
"""

__all__ = ['Experiment', ]


class Experiment:
    """Base class of experiments."""
