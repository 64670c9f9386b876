"""Import shim: `import ernn_gb300` loads the package that lives in the
directory elastodynamics-encoded-rnn_gb300/ (a name Python cannot import
directly because of its hyphens)."""
import importlib.util as _ilu
import os as _os
import sys as _sys

_root = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "elastodynamics-encoded-rnn_gb300")
_spec = _ilu.spec_from_file_location(__name__, _os.path.join(_root, "__init__.py"),
                                     submodule_search_locations=[_root])
_mod = _ilu.module_from_spec(_spec)
_sys.modules[__name__] = _mod
_spec.loader.exec_module(_mod)
