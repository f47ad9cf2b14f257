"""Import the unmodified PETITE reference in the development container.

Used only by the fixture-generating scripts in this directory (never by the
engine, the oracle or the GPU tests).  PETITE needs ``vegas`` and
``matplotlib`` at import time; neither is installed, so the project-written
shims in ``refshim/`` are put first on ``sys.path``.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("PETITE_REFERENCE", "/root/reference")


def setup():
    for p in (os.path.join(HERE, "refshim"), os.path.join(REFERENCE, "src"),
              os.path.join(REFERENCE, "utilities")):
        if p not in sys.path:
            sys.path.insert(0, p)
    if not os.path.isdir(os.path.join(REFERENCE, "src", "PETITE")):
        raise RuntimeError(f"PETITE reference not found under {REFERENCE}")
