"""Bridge between models and interactive front-ends (reference ``xentica/bridge``).

Only the action table is provided; the Moire GUI itself (OpenGL/Kivy) is an
external application.
"""
from xentica_gb300.bridge.moire import MoireBridge

__all__ = ["MoireBridge", ]
