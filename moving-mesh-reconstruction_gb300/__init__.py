"""GB300-native (sm_103a) MMH reconstruction hot path.

The package directory name is not a Python identifier; load it with
importlib.import_module("moving-mesh-reconstruction_gb300") or put the
directory on sys.path and import the modules mmh, fields, build.
"""
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
if _HERE not in sys.path:
    sys.path.insert(0, _HERE)

import build  # noqa: E402,F401
import fields  # noqa: E402,F401
import mmh  # noqa: E402,F401
from mmh import Context, MMHError, reconstruct  # noqa: E402,F401
