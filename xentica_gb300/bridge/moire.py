"""Key actions for the Moire front-end (reference ``xentica/bridge/moire.py``).

``[`` slower, ``]`` faster, space pause, F12 system info, Esc exit; renderers
add their own keys (move and zoom for ``RendererPlain``).
"""
from xentica_gb300.bridge.base import Bridge

__all__ = ['MoireBridge', ]


class MoireBridge:
    """Key-to-action table."""

    key_actions = {
        "[": Bridge.speed(-1),
        "]": Bridge.speed(1),
        "spacebar": Bridge.toggle_pause,
        "f12": Bridge.toggle_sysinfo,
        "escape": Bridge.exit_app,
    }
