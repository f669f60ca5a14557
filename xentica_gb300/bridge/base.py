"""Generic bridge actions (reference ``xentica/bridge/base.py:11-39``).

Every action is a callable ``action(model, gui)``.
"""

__all__ = ['Bridge', ]


class Bridge:
    """Basic actions shared by all bridges."""

    @staticmethod
    def noop(_model, _gui):
        """Do nothing."""

    @staticmethod
    def exit_app(_model, gui):
        """Ask the GUI to exit."""
        gui.exit_app()

    @staticmethod
    def speed(dspeed):
        """Action changing the simulation speed by ``dspeed``."""
        def func(model, _gui):
            model.apply_speed(dspeed)
        return func

    @staticmethod
    def toggle_pause(model, _gui):
        """Pause or resume the simulation."""
        model.toggle_pause()

    @staticmethod
    def toggle_sysinfo(_model, gui):
        """Show or hide the GUI's system-info panel."""
        gui.sysinfo.toggle()
