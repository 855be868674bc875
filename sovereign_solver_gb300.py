"""Import name for the ``sovereign-solver_gb300/`` package directory.

The package directory carries a hyphen, which Python's import statement cannot
spell.  Importing ``sovereign_solver_gb300`` executes this file, which loads the
directory as a regular package under this name and replaces itself in
``sys.modules`` so that ``import sovereign_solver_gb300.pdhg`` and friends
resolve inside the directory.
"""

import importlib.util
import os
import sys

_PKG_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sovereign-solver_gb300")
_spec = importlib.util.spec_from_file_location(
    __name__,
    os.path.join(_PKG_DIR, "__init__.py"),
    submodule_search_locations=[_PKG_DIR],
)
_pkg = importlib.util.module_from_spec(_spec)
sys.modules[__name__] = _pkg
_spec.loader.exec_module(_pkg)
