"""Drop-in for the reference's ``libhbvlm3`` pybind module: put this
directory on ``sys.path`` and ``from libhbvlm3 import HBVLM`` as before."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
from tinyvlm_gb300.hbvlm import HBVLM3 as HBVLM  # noqa: E402,F401
