"""CPU checks of the C-ABI boundary: the library loads and exports every
symbol include/fsim.h declares; the binding declares no extra symbol; the
host-only dt rule matches the oracle's restatement."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "fsim.h"


def declared_symbols():
    txt = HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fsim_[a-z0-9_]+)\s*\(", txt)))


def _lib():
    import fsim

    if not fsim.LIB_PATH.exists():
        pytest.skip("libfsim.so not built (nvcc unavailable)")
    return fsim.load_library()


def test_library_exports_every_declared_symbol():
    lib = _lib()
    syms = declared_symbols()
    assert len(syms) >= 35
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    import fsim

    assert sorted(fsim._SIGS) == declared_symbols()


def test_version_and_null_handle():
    lib = _lib()
    assert b"sm_103a" in lib.fsim_version()
    assert lib.fsim_last_error(None) == b"null handle"
    assert lib.fsim_destroy(None) == 0


def test_create_rejects_bad_config_without_gpu_work():
    import fsim

    lib = _lib()
    cfg = fsim.fsim_config()
    for d in range(3):
        cfg.global_dims[d] = 4  # below the 8-cell minimum
    cfg.nparticles_per_cell = 8
    h = ctypes.c_void_p()
    assert lib.fsim_create(ctypes.byref(cfg), ctypes.byref(h)) == fsim.ERR_INVALID


def test_compute_dt_matches_oracle_rule():
    import fsim
    from oracle.oracle import compute_dt

    fs = float(np.float32(1) / np.float32(30))
    rng = np.random.default_rng(3)
    for inv in list(rng.uniform(1e-4, 0.2, 200)) + [1e-6, 0.5, 10.0]:
        for t in (0.0, 0.01, 0.03, 0.0333):
            a = fsim.compute_dt(float(inv), 1, fs, t)
            b = compute_dt(float(inv), 1, fs, t)
            assert a[0] == pytest.approx(b[0], abs=0) and a[1] == b[1]


def test_struct_layouts_match_header(tmp_path):
    """Compile the header with the system C compiler and compare every
    struct's size and field offsets with the ctypes mirror."""
    import shutil
    import subprocess

    import fsim

    if not shutil.which("gcc"):
        pytest.skip("gcc unavailable")
    structs = [fsim.fsim_config, fsim.fsim_shape, fsim.fsim_seed_pass, fsim.fsim_pcg_params,
               fsim.fsim_pcg_stats, fsim.fsim_step_stats, fsim.fsim_source, fsim.fsim_scene,
               fsim.fsim_run_stats]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fsim.h"', "int main(void){"]
    for st in structs:
        n = st.__name__
        lines.append(f'printf("{n} %zu\\n", sizeof({n}));')
        for f in st._fields_:
            lines.append(f'printf("{n}.{f[0]} %zu\\n", offsetof({n}, {f[0]}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True,
                                                          text=True, check=True).stdout.split("\n") if l)
    for st in structs:
        n = st.__name__
        assert int(out[n]) == ctypes.sizeof(st), n
        for f in st._fields_:
            assert int(out[f"{n}.{f[0]}"]) == getattr(st, f[0]).offset, (n, f[0])
