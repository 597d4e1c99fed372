"""The C-ABI library builds, loads and exports every symbol include/bhk.h declares (no compute)."""
import ctypes
import os
import subprocess

import pytest

from black_simulation_gb300 import bhk, build


@pytest.fixture(scope="module")
def libbhk():
    build.build()
    return bhk.lib()


def test_every_declared_symbol_is_exported(libbhk):
    declared = bhk.exported_symbols()
    assert len(declared) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", bhk.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing


def test_version_and_flop_count(libbhk):
    assert b"sm_103a" in libbhk.bhk_version()
    assert bhk.flops_per_step() > 100
    # a rejected attempt runs the stages and the error norm, not the accepted step's tail
    assert 0.9 * bhk.flops_per_step() < bhk.flops_per_rejected_step() < bhk.flops_per_step()


def test_struct_layouts_match_header():
    assert ctypes.sizeof(bhk.FrameDescC) == 4 * 8 + 2 * 4 + 6 * 8
    assert ctypes.sizeof(bhk.RaysOutC) == 15 * 8  # 8 core + 7 optional RayReport fields


def test_no_cpu_fallback_without_gpu(libbhk):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = libbhk.bhk_create(0, ctypes.byref(h))
    assert st == bhk.ECUDA
    assert b"no CUDA device" in libbhk.bhk_last_error()


def test_invalid_arguments_rejected_before_any_launch(libbhk):
    # Null arrays with n > 0 are EINVAL; n == 0 is a no-op (the reference's empty loops).
    assert libbhk.bhk_step_mino(0.9, None, None, None, 4, None) == bhk.EINVAL
    assert libbhk.bhk_step_mino(0.9, None, None, None, 0, None) == bhk.OK
    assert libbhk.bhk_normalize_angles(None, -1, None) == bhk.EINVAL
    assert libbhk.bhk_trace_frames(None, None, 0, None, None, None) == bhk.EINVAL


def test_library_is_in_tree():
    assert os.path.dirname(bhk.LIB_PATH).endswith("black_simulation_gb300")
