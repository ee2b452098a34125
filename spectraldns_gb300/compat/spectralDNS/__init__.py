"""spectralDNS import name resolved to the GB300 backend."""
import sys

import spectraldns_gb300 as _gb
from spectraldns_gb300 import config, get_solver, solve  # noqa: F401
from spectraldns_gb300 import utilities  # noqa: F401

sys.modules[__name__ + ".config"] = _gb.config
sys.modules[__name__ + ".utilities"] = _gb.utilities
__version__ = _gb.__version__
