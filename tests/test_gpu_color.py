"""Bit-exactness of the guide colour conversion (a1) over all 2^24 RGB
triples, and the pin of the oracle's evaluation order against nvcc."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PROBE = Path(__file__).resolve().parent / "probes" / "color_expr_probe.cu"


def _all_pixels(alpha=7):
    idx = np.arange(1 << 24, dtype=np.uint32)
    px = np.empty((1 << 24, 4), np.uint8)
    px[:, 0] = idx >> 16
    px[:, 1] = (idx >> 8) & 255
    px[:, 2] = idx & 255
    px[:, 3] = alpha
    return px


def test_reference_expression_order_pins_the_oracle(gpu_ready, oracle_mod, tmp_path):
    """nvcc-compiled reference expression == the oracle's default order, and
    differs from the other candidate orders (so the pin is informative)."""
    so = tmp_path / "probe.so"
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                    "-shared", "-Xcompiler", "-fPIC", "-o", str(so), str(PROBE)],
                   check=True)
    lib = ctypes.CDLL(str(so))
    lib.probe_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    px = _all_pixels()
    out = np.empty_like(px)
    assert lib.probe_run(px.ctypes.data, out.ctypes.data, px.shape[0]) == 0
    matches = {}
    for order in (0, 1, 2):
        ref = oracle_mod.color_convert(1, px, contract=order)
        matches[order] = int((ref != out).any(1).sum())
    assert matches[oracle_mod.DEFAULT_CONTRACT] == 0, matches
    assert all(v > 0 for k, v in matches.items() if k != oracle_mod.DEFAULT_CONTRACT)


@pytest.mark.parametrize("cs", [0, 1, 2])
def test_product_kernel_exhaustive(gpu_ready, oracle_mod, cs):
    from domain_transform_solver_gb300 import _lib
    lib = _lib.load()
    px = _all_pixels()
    out = np.empty_like(px)
    _lib.check(lib.dtsgb_debug_color_convert(cs, px.ctypes.data, out.ctypes.data,
                                             px.shape[0]))
    ref = oracle_mod.color_convert(cs, px)
    bad = (ref != out).any(1)
    assert bad.sum() == 0, np.nonzero(bad)[0][:10]
