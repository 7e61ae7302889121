"""Spherical Bessel transforms (jrystal/sbt): the numerical transform the
pseudopotential tables are built from, under the reference's name
``sbt_numerical`` (jrystal/sbt/sbt_numerical.py:13-81).  The log-grid fast
transform (pysbt) is not part of this package."""
from .pseudopotential.sbt import sbt as sbt_numerical  # noqa: F401

__all__ = ["sbt_numerical"]
