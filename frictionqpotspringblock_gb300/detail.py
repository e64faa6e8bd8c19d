"""The reference's `detail` submodule as far as Python sees it (main.cpp:246-275): the class of
`system.external` of the RandomForcing systems."""

from ._system import RandomNormalForcing as RandomNormalForcing_1  # noqa: F401
