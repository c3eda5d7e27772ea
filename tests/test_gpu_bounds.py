"""The bounds-check build (libnerfgb_bounds.so, compiled with
-DNERF_BOUNDS_CHECK): every index the kernels compute from data is checked
against its buffer (csrc/common.cuh, NG_IDX). The small-shape parity cases of
the samplers, gates and fused render run on it in a child process, which then
reads nerfgb_bounds_check_status: no check may have failed. A row map with a
row past the end shows that a failing check is recorded (the index is clamped
in bounds, so the read stays inside the buffer)."""
import os
import pathlib
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = pathlib.Path(__file__).resolve().parent.parent
BOUNDS_LIB = ROOT / "nerf-tf2_gb300" / "libnerfgb_bounds.so"

CHILD = r"""
import ctypes, importlib, sys
import pytest
rc = pytest.main(["-q", "-m", "gpu", "-p", "no:cacheprovider", "-x",
                  "tests/test_gpu_ray_ops.py", "tests/test_gpu_gate.py", "tests/test_gpu_render.py",
                  "-k", "not quality and not lowp and not 1024"])
ng = importlib.import_module("nerf-tf2_gb300")
lib = ng._lib.lib()
status = lib.nerfgb_bounds_check_status(1)
print("BOUNDS_STATUS", status, flush=True)
if rc != 0 or status != 0:
    sys.exit(1)
# a failing check is recorded: row 10 of a 4-row MLP input through the row map
import torch
X = torch.zeros(4, 3, device="cuda"); D = torch.zeros(4, 3, device="cuda")
mp = torch.tensor([0, 1, 10, 2], dtype=torch.int32, device="cuda")
rgb = torch.zeros(4, 3, device="cuda"); sig = torch.zeros(4, device="cuda")
mlp = ng.get_coarse_or_fine_model("fine", seed=1, precision="fp32")
ng._lib.call("nerfgb_mlp_forward_mapped", mlp.packed().data_ptr(), ng._lib.PREC_FP32, X.data_ptr(), D.data_ptr(),
             4, 1, mp.data_ptr(), None, rgb.data_ptr(), sig.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
torch.cuda.synchronize()
planted = lib.nerfgb_bounds_check_status(1)
print("PLANTED_STATUS", planted, flush=True)
sys.exit(0 if planted == 9 and lib.nerfgb_bounds_check_status(1) == 0 else 2)
"""


def test_parity_cases_on_the_bounds_check_build(ng, cuda):
    assert BOUNDS_LIB.exists(), "build() makes libnerfgb_bounds.so beside libnerfgb.so"
    # the library this process loaded is the normal build
    assert ng._lib.lib().nerfgb_bounds_check_status(0) == ng._lib.E_UNSUPPORTED
    env = dict(os.environ, NERFGB_LIBRARY=str(BOUNDS_LIB))
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=str(ROOT), env=env, capture_output=True, text=True,
                       timeout=900)
    tail = (r.stdout + r.stderr)[-3000:]
    assert "BOUNDS_STATUS 0" in r.stdout, tail
    assert r.returncode == 0, tail
