"""Utilities mirrored from chromo.util that the MC loop needs."""
