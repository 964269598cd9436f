"""CPU checks of the drop-in boundary: libdtsgb.so builds for sm_103a, loads
without a GPU, and exports every entry point include/dtsgb.h declares.  No
compute call is made here."""
import ctypes

from domain_transform_solver_gb300 import _lib


def test_header_declares_the_reference_surface():
    names = set(_lib.declared_symbols())
    for n in ["dtsgb_dts_create", "dtsgb_dts_init_frame", "dtsgb_dts_optimize",
              "dtsgb_dts_filter", "dtsgb_dts_compute_confidence",
              "dtsgb_dts_download", "dtsgb_dts_clear_all",
              "dtsgb_dts_set_image_dim", "dtsgb_dts_compute_differential",
              "dtsgb_dts_integrate", "dtsgb_hfbs_create", "dtsgb_hfbs_init_frame",
              "dtsgb_hfbs_set_filter_params", "dtsgb_hfbs_optimize",
              "dtsgb_hfbs_download", "dtsgb_hfbs_clear_all",
              "dtsgb_hfbs_set_image_dim", "dtsgb_last_error"]:
        assert n in names


def test_library_exports_every_declared_symbol(dts):
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in _lib.declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_error_string_before_any_call(dts):
    lib = _lib.load()
    assert lib.dtsgb_version() >= 1
    # a null handle is rejected without touching the GPU
    assert lib.dtsgb_dts_set_image_dim(None, 10, 10) == _lib.DTSGB_ERR_INVALID_ARGUMENT
    assert b"null" in lib.dtsgb_last_error()
    assert lib.dtsgb_hfbs_optimize(None) == _lib.DTSGB_ERR_INVALID_ARGUMENT
    assert lib.dtsgb_dts_create(0, 10, 0, None) == _lib.DTSGB_ERR_INVALID_ARGUMENT


def test_gradient_entry_points_reject_null_handles(dts):
    """The HFBS gradient calls validate their arguments before any CUDA call."""
    lib = _lib.load()
    bad = _lib.DTSGB_ERR_INVALID_ARGUMENT
    assert lib.dtsgb_hfbs_enable_grad(None, 1, 0) == bad
    assert lib.dtsgb_hfbs_grad_info(None, None, None) == bad
    assert lib.dtsgb_hfbs_backward(None, None, None, None) == bad
    assert lib.dtsgb_hfbs_backward_device(None, None, None, None) == bad
    assert lib.dtsgb_batch_hfbs_backward(None, None, None, None) == bad
    assert lib.dtsgb_batch_hfbs_backward_device(None, None, None, None) == bad
    assert lib.dtsgb_batch_hfbs_grad_info(None, None, None) == bad


def test_bench_names_every_profiler_kind():
    """bench.py reports every kernel kind the header's profiler enum holds
    (DTSGB_K_* below DTSGB_K_COUNT), each under its own name."""
    import ast
    import re
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    header = (root / "include" / "dtsgb.h").read_text()
    kinds = {int(v) for n, v in re.findall(r"\b(DTSGB_K_\w+)\s*=\s*(\d+)", header)
             if n != "DTSGB_K_COUNT"}
    count = int(re.search(r"DTSGB_K_COUNT\s*=\s*(\d+)", header).group(1))
    assert kinds == set(range(count))
    tree = ast.parse((root / "bench.py").read_text())
    names = next(ast.literal_eval(node.value) for node in tree.body
                 if isinstance(node, ast.Assign)
                 and any(getattr(t, "id", None) == "KERNEL_NAMES" for t in node.targets))
    assert set(names) == kinds
    assert len(set(names.values())) == len(names)
