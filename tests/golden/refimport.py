"""Import the unmodified PETITE reference in the development container.

Used only by the fixture-generating scripts in this directory (never by the
engine, the oracle or the GPU tests).  PETITE needs ``vegas`` and
``matplotlib`` at import time; neither is installed, so the project-written
shims in ``refshim/`` are put first on ``sys.path``.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the PETITE checkout (the directory holding src/PETITE), given by the caller
REFERENCE = os.environ.get("PETITE_REFERENCE", "")


def setup():
    if not REFERENCE:
        raise RuntimeError("set PETITE_REFERENCE to a PETITE checkout (the directory holding src/PETITE)")
    for p in (os.path.join(HERE, "refshim"), os.path.join(REFERENCE, "src"),
              os.path.join(REFERENCE, "utilities")):
        if p not in sys.path:
            sys.path.insert(0, p)
    if not os.path.isdir(os.path.join(REFERENCE, "src", "PETITE")):
        raise RuntimeError(f"PETITE reference not found under {REFERENCE}")
