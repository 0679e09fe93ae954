"""A compiled C program calls the library through include/bhgpu.h, as the reference app would
(tests/c_caller/app_frame.c: the app's 80-byte Body records in and out, a few frames of bh_step).
Without a GPU the program must get BH_ERR_DEVICE from bh_create and stop cleanly; on a GPU it
runs the frames."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "serial-hashed-octree-barnes-hut-n-body-simulator-0_3_gb300")
SRC = os.path.join(ROOT, "tests", "c_caller", "app_frame.c")


def _compile(bh, tmp_path):
    bh.load()  # builds libbhgpu.so if needed
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "app_frame")
    cmd = [cc, "-std=c99", "-Wall", "-Werror", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", PKG, "-lbhgpu", "-Wl,-rpath," + PKG, "-lm"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    return exe


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def test_c_caller_without_gpu_gets_device_error(bh, tmp_path):
    if _has_gpu():
        pytest.skip("a GPU is visible: the GPU test below runs the frames")
    exe = _compile(bh, tmp_path)
    out = subprocess.run([exe, "4444", "3"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 10, out.stdout + out.stderr
    assert "bh_create -> 3" in out.stdout


@pytest.mark.gpu
def test_c_caller_runs_app_frames(bh, tmp_path):
    exe = _compile(bh, tmp_path)
    out = subprocess.run([exe, "4444", "3"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "ok n=4444 frames=3" in out.stdout
