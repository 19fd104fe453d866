"""Load the ``halign-4_gb300`` package directory as the module ``halign_gb300``.

The directory name carries a hyphen, so it cannot be imported by name; tests,
bench.py and the entry point load it through this helper.
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "halign-4_gb300"


def load_package():
    mod = sys.modules.get("halign_gb300")
    if mod is not None:
        return mod
    spec = importlib.util.spec_from_file_location("halign_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["halign_gb300"] = mod
    spec.loader.exec_module(mod)
    import halign_gb300.autotune  # noqa: F401  (attach the submodules)
    import halign_gb300.serve  # noqa: F401
    import halign_gb300.shard  # noqa: F401
    import halign_gb300.synth  # noqa: F401
    return mod
