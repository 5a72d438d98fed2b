"""Optional third-party modules, imported only when present.

Same contract as the reference's python/python/rusterize/_dependencies.py:
each name is either the real module or a placeholder that raises
ModuleNotFoundError on attribute access, plus availability predicates.
"""

from __future__ import annotations

import importlib.util
import sys
from functools import cache
from typing import Any


class _Missing:
    def __init__(self, name: str):
        self._name = name

    def __getattr__(self, attr: str) -> Any:
        raise ModuleNotFoundError(f"{attr} requires the {self._name!r} module to be installed.")


def _optional(name: str) -> tuple[Any, bool]:
    if name in sys.modules:
        return sys.modules[name], True
    try:
        spec = importlib.util.find_spec(name)
    except (ModuleNotFoundError, ValueError):
        spec = None
    if spec is None or spec.loader is None:
        return _Missing(name), False
    spec.loader = importlib.util.LazyLoader(spec.loader)
    module = importlib.util.module_from_spec(spec)
    sys.modules[name] = module
    spec.loader.exec_module(module)
    return module, True


geopandas, GEOPANDAS_AVAILABLE = _optional("geopandas")
polars, POLARS_AVAILABLE = _optional("polars")
polars_st, POLARS_ST_AVAILABLE = _optional("polars_st")
xarray, XARRAY_AVAILABLE = _optional("xarray")
_rioxarray, RIOXARRAY_AVAILABLE = _optional("rioxarray")
shapely, SHAPELY_AVAILABLE = _optional("shapely")


def _xarray_available() -> bool:
    return XARRAY_AVAILABLE and RIOXARRAY_AVAILABLE


def _polars_available() -> bool:
    return POLARS_AVAILABLE


@cache
def _mro_mentions(cls: type, module: str) -> bool:
    try:
        return any(f"{module}." in str(o) for o in cls.mro())
    except TypeError:
        return False


def _check_for_geopandas(obj: Any) -> bool:
    return GEOPANDAS_AVAILABLE and _mro_mentions(type(obj), "geopandas")


def _check_for_polars_st(obj: Any) -> bool:
    return POLARS_ST_AVAILABLE and _mro_mentions(type(obj), "polars")
