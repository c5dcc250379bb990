"""The C-ABI library: builds, loads without a GPU, exports every declared entry
point, and its config struct has the layout the Python binding assumes."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from pbi4_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pbi4gpu.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pbi4g_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.lib()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.EXPORTS)


def test_no_other_symbols_exported():
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True).stdout
    funcs = {l.split()[-1] for l in out.splitlines() if " T " in l}
    ours = {f for f in funcs if f.startswith("pbi4g_")}
    assert ours == set(declared())


def test_config_struct_layout(tmp_path):
    c = tmp_path / "t.c"
    c.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "pbi4gpu.h"\n'
                 'int main(void){printf("%zu %zu %zu %zu\\n", sizeof(pbi4g_config), offsetof(pbi4g_config, los),'
                 ' offsetof(pbi4g_config, precision), offsetof(pbi4g_config, reserved));'
                 'printf("%zu\\n", offsetof(pbi4g_config, map_budget_mb));return 0;}\n')
    exe = tmp_path / "t"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    C = _lib.Config
    want = [ctypes.sizeof(C), C.los.offset, C.precision.offset, C.reserved.offset, C.map_budget_mb.offset]
    assert [int(x) for x in got] == want


def test_errors_without_device(lib):
    """Argument validation happens before any device work, so it answers on a CPU-only host."""
    cfg = _lib.Config()
    cfg.grid = 7  # odd grid: rejected
    out = ctypes.c_int64()
    rc = lib.pbi4g_plan_footprint(ctypes.byref(cfg), 10, ctypes.byref(out))
    assert rc == 1
    assert b"grid" in lib.pbi4g_last_error()
    cfg.grid, cfg.box, cfg.nintp, cfg.nbins_ps, cfg.kbin_ps = 256, 1000.0, 4, 128, 1.0
    assert lib.pbi4g_plan_footprint(ctypes.byref(cfg), 2 ** 21, ctypes.byref(out)) == 0
    assert out.value > 256 ** 3 * 8


def test_scratch_footprint_without_device(lib):
    """The shared assignment scratch's size is the plan's own record buffers'
    (a plan that shares one leaves exactly that much out), and bad arguments are
    rejected on the host."""
    out = ctypes.c_int64()
    assert lib.pbi4g_scratch_footprint(1024, 10 ** 7, 0, ctypes.byref(out)) == 0
    # 32-byte particle record, up to 8 tile records of 32 bytes and their weights
    records = 3 * ((1024 // 16) ** 3 + 2) * 4 + 10 ** 7 * (32 + 8 * (32 + 4)) + 64
    assert out.value == records
    assert lib.pbi4g_scratch_footprint(1024, 10 ** 7, 4, ctypes.byref(out)) == 0
    assert out.value == records + 4 * 3 * 10 ** 7 * 8  # and four graph position slots
    assert lib.pbi4g_scratch_footprint(40, 1000, 0, ctypes.byref(out)) == 1  # not a multiple of 16
    assert lib.pbi4g_scratch_footprint(64, 0, 0, ctypes.byref(out)) == 1
    assert lib.pbi4g_scratch_footprint(64, 1000, -1, ctypes.byref(out)) == 1
    assert b"scratch" in lib.pbi4g_last_error()


@pytest.mark.parametrize("n", [2, 3, 5, 7, 8, 12, 20, 40, 50, 60, 100, 128, 140, 150, 196, 200, 240, 294, 320,
                               392, 400, 480, 512, 640, 8000])
def test_fft_plan_host(lib, n):
    """The in-place mixed-radix plans of the shell-map transforms (radices 2, 3,
    4, 5, 7, 8, 10 and 20; digit-reversed output positions) against numpy's
    inverse DFT."""
    import numpy as np
    rng = np.random.default_rng(n)
    batch = 3
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    out = np.zeros_like(x)
    rc = lib.pbi4g_fft_plan_check(n, batch, x.ctypes.data, out.ctypes.data)
    assert rc == 0, lib.pbi4g_last_error()
    ref = np.fft.ifft(x.astype(np.complex128), axis=1) * n
    assert np.max(np.abs(out - ref)) <= 1e-6 * np.max(np.abs(ref))


def test_fft_plan_rejects_large_primes(lib):
    import numpy as np
    x = np.zeros(22, dtype=np.complex64)
    for n in (11, 22, 26):
        assert lib.pbi4g_fft_plan_check(n, 1, x.ctypes.data, x.ctypes.data) != 0
        assert b"fft plan" in lib.pbi4g_last_error()
