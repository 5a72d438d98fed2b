"""Optional third-party libraries of the Python front end.

The front end accepts GeoPandas and polars-st inputs and can return xarray
rasters or polars frames, but it burns without any of those libraries.  Each
one is represented here by an ``OptionalModule``: a proxy that imports the
library the first time one of its attributes is used, and raises
ModuleNotFoundError naming the library when it is not installed.  The
predicates below tell the front end which input types can occur and which
encodings can be produced, without importing anything.
"""

from __future__ import annotations

import importlib
import importlib.util
from typing import Any


class OptionalModule:
    """Stand-in for an importable-if-installed module."""

    __slots__ = ("_name", "_installed", "_module")

    def __init__(self, name: str):
        self._name = name
        self._installed: bool | None = None
        self._module = None

    @property
    def installed(self) -> bool:
        if self._installed is None:
            try:
                self._installed = importlib.util.find_spec(self._name) is not None
            except (ImportError, ValueError):
                self._installed = False
        return self._installed

    def load(self, what: str = "") -> Any:
        """The module itself, imported on first use."""
        if self._module is None:
            if not self.installed:
                need = f" (needed for {self._name}.{what})" if what else ""
                raise ModuleNotFoundError(f"the optional dependency {self._name!r} is not installed{need}",
                                          name=self._name)
            self._module = importlib.import_module(self._name)
        return self._module

    def __getattr__(self, attr: str) -> Any:
        return getattr(self.load(attr), attr)


geopandas = OptionalModule("geopandas")
polars = OptionalModule("polars")
polars_st = OptionalModule("polars_st")
xarray = OptionalModule("xarray")
rioxarray = OptionalModule("rioxarray")
shapely = OptionalModule("shapely")


def _xarray_available() -> bool:
    """encoding="xarray" needs xarray and the rioxarray accessor (for the CRS)."""
    return xarray.installed and rioxarray.installed


def _polars_available() -> bool:
    return polars.installed


def _class_from(obj: Any, package: str) -> bool:
    """Whether the type of obj, or one of its bases, is defined in `package`."""
    for cls in type(obj).__mro__:
        mod = getattr(cls, "__module__", "") or ""
        if mod == package or mod.startswith(package + "."):
            return True
    return False


def _check_for_geopandas(obj: Any) -> bool:
    return geopandas.installed and _class_from(obj, "geopandas")


def _check_for_polars_st(obj: Any) -> bool:
    """A polars frame (polars-st keeps its geometries in polars frames)."""
    return polars_st.installed and _class_from(obj, "polars")
