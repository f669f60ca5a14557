"""Helpers used inside model definitions."""

from .xmath import Xmath as xmath

__all__ = ["xmath", ]
