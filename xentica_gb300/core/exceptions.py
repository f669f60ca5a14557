"""Framework exception (reference ``xentica/core/exceptions.py:6-7``)."""

__all__ = ['XenticaException', ]


class XenticaException(Exception):
    """The basic framework exception."""
