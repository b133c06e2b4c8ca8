"""Drop-in for the reference's ``libhbvlm`` pybind module (2-DOF): put this
directory on ``sys.path`` and ``from libhbvlm import HBVLM`` as before."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
from tinyvlm_gb300.hbvlm import HBVLM2 as HBVLM  # noqa: E402,F401
