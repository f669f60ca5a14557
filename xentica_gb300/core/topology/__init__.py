"""Lattices, neighbourhoods and borders (reference ``xentica/core/topology``)."""
