"""petite_gb300 -- GB300-native electromagnetic-shower engine, a drop-in for
PETITE's Shower/DarkShower transport path (kjkellyphys/PETITE).

The transport runs in hand-written sm_103a CUDA kernels (``csrc/``) behind
the C ABI in ``include/petite_gpu.h``; this package is the host side:
tables (``tables``), the device engine (``engine``), and the PETITE-shaped
API (``Particle``, ``Shower``, ``DarkShower``).
"""
from .particle import Particle
from .shower import Shower, ShowerBatch, list_order
from .dark import DarkShower
from .tables import BUNDLED_DIR, PROCESSES, TARGET_INFORMATION

__all__ = ["Particle", "Shower", "ShowerBatch", "DarkShower", "list_order", "BUNDLED_DIR", "PROCESSES",
           "TARGET_INFORMATION"]
__version__ = "0.1.0"
