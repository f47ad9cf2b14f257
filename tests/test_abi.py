"""The C ABI without a GPU: every function declared in include/*.h is exported
by the built library and bound by the ctypes layer, and the ctypes structures
have the header's layout (offsets checked against a gcc-compiled probe)."""
import ctypes as C
import glob
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = sorted(glob.glob(os.path.join(ROOT, "include", "*.h")))


def declared_functions():
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w ]*?[\s*]+(pt_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return names


def test_header_declares_the_bound_exports():
    from petite_gb300 import _lib
    names = declared_functions()
    assert len(names) == len(set(names))
    assert set(names) == set(_lib.EXPORTS)


@pytest.fixture(scope="module")
def lib():
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not available")
    from petite_gb300 import _lib
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_strerror_needs_no_device(lib):
    from petite_gb300 import _lib
    assert lib.pt_strerror(_lib.PT_NO_SAMPLE) == b"No Sample Found"
    assert lib.pt_strerror(_lib.PT_OK) == b"ok"
    assert lib.pt_strerror(99) == b"unknown status"


def test_struct_layout_matches_header(tmp_path):
    """Offsets of every field of the ABI structures, from gcc on the header,
    against the ctypes definitions."""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    from petite_gb300 import _lib
    structs = {"pt_tables": _lib.PtTables, "pt_particles": _lib.PtParticles, "pt_opts": _lib.PtOpts,
               "pt_tally": _lib.PtTally, "pt_dark_maps": _lib.PtDarkMaps, "pt_dark_params": _lib.PtDarkParams,
               "pt_dark_out": _lib.PtDarkOut, "pt_batch_tuning": _lib.PtBatchTuning,
               "pt_train_target": _lib.PtTrainTarget, "pt_dark_hist": _lib.PtDarkHist}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "petite_gpu.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f.rstrip("_")}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {(a, b): int(c) for a, b, c in (ln.split() for ln in out if ln)}
    for cname, cls in structs.items():
        assert got[(cname, "sizeof")] == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_entry_points_refuse_missing_handles_without_a_device(lib):
    """Argument checks that return before any CUDA call: null handles and
    out-of-range counts give PT_BAD_ARG on a machine without a GPU."""
    from petite_gb300 import _lib
    i64 = C.c_int64()
    opts, tally, prm = _lib.PtOpts(), _lib.PtTally(), _lib.PtDarkParams()
    assert lib.pt_run_batch(None, None, None, None, None, 1, C.byref(opts), C.byref(tally), 0, None) == _lib.PT_BAD_ARG
    assert lib.pt_run_batch_dark(None, None, C.byref(prm), 1, None, None, None, None, 1, C.byref(opts),
                                 C.byref(tally), 0, None, None, None, C.byref(i64), None) == _lib.PT_BAD_ARG
    assert lib.pt_dark_screen32(None, 0, None, None, 1, 0.1, None, None, None) == _lib.PT_BAD_ARG
    assert lib.pt_set_batch_tuning(None, None) == _lib.PT_BAD_ARG
    assert lib.pt_vegas_adapt(0, 1, None, None, 2, None, None, 0.5, None) == _lib.PT_BAD_ARG
    assert lib.pt_detector_cut(None, 0, None, 0, None, 5, None, 1, 0.0, 1.0, 0, 0.0, 0.0, None, None,
                               None) == _lib.PT_BAD_ARG
    buf = (C.c_double * 64)()
    # strides shorter than the rows, a negative count, detectors without positions
    assert lib.pt_detector_cut(buf, 4, buf, 8, None, 8, buf, 1, 0.0, 1.0, 0, 0.0, 0.0, None, None,
                               None) == _lib.PT_BAD_ARG
    assert lib.pt_detector_cut(buf, 8, buf, 8, None, -1, buf, 1, 0.0, 1.0, 0, 0.0, 0.0, None, None,
                               None) == _lib.PT_BAD_ARG
    assert lib.pt_detector_cut(buf, 8, buf, 8, None, 8, None, 2, 0.0, 1.0, 0, 0.0, 0.0, None, None,
                               None) == _lib.PT_BAD_ARG


def test_staging_timeout_marks_the_handle_unusable():
    """PT_TIMEOUT whose error record names a table-staging copy (process -2)
    makes the engine refuse further device work: that copy may still be in
    flight.  A loop bound (process -1) does not."""
    from petite_gb300 import _lib
    from petite_gb300.engine import SMEngine

    class FakeLib:
        def __init__(self, proc):
            self.proc = proc

        def pt_last_error_info(self, h, proc, E, key):
            C.cast(proc, C.POINTER(C.c_int32))[0] = self.proc
            return 0

    for proc, unusable in ((-1, False), (-2, True)):
        eng = object.__new__(SMEngine)
        eng.unusable = None
        eng.handle = None
        eng.lib = FakeLib(proc)
        with pytest.raises(_lib.PetiteGPUError):
            eng._raise(_lib.PT_TIMEOUT, "pt_run_batch")
        assert (eng.unusable is not None) == unusable
        if unusable:
            with pytest.raises(_lib.PetiteGPUError):
                eng._usable()
