"""The command-line driver's frame writer pool (worker threads converting,
encoding and writing frames, recycled frame buffers, a bounded queue), run on
the host through a small harness that includes the driver's source: every
frame is read back and equals the byte conversion of what was submitted."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "probabilistic_fluid_simulation_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "png_writers_main.cpp")


@pytest.fixture(scope="module")
def harness(tmp_path_factory, pfs_lib):
    exe = str(tmp_path_factory.mktemp("bin") / "png_writers_main")
    cmd = ["g++", "-O2", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(PKG, "cli"), SRC, os.path.join(PKG, "cli", "png.cpp"), "-o", exe, "-L", PKG,
           "-lpfs_gb300", f"-Wl,-rpath,{PKG}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("frames,w,h,threads,queue", [(40, 64, 48, 4, 2), (9, 33, 7, 1, 1), (25, 128, 96, 8, 16)])
def test_frames_written_in_order_and_intact(harness, tmp_path, frames, w, h, threads, queue):
    r = subprocess.run([harness, str(tmp_path), str(frames), str(w), str(h), str(threads), str(queue)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == f"ok {frames} frames"
    assert sorted(os.listdir(tmp_path)) == sorted(f"{f}.png" for f in range(frames))


def test_writer_pool_has_no_data_races(tmp_path, pfs_lib):
    """The same harness under ThreadSanitizer: the queue, the buffer free
    list, the error slot and the codec's shared tables are race-free."""
    exe = str(tmp_path / "png_writers_tsan")
    cmd = ["g++", "-O1", "-g", "-std=c++17", "-fsanitize=thread", "-pthread", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(PKG, "cli"), SRC, os.path.join(PKG, "cli", "png.cpp"), "-o", exe, "-L", PKG,
           "-lpfs_gb300", f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("ThreadSanitizer not available")
    assert r.returncode == 0, r.stderr
    out = tmp_path / "frames"
    out.mkdir()
    r = subprocess.run([exe, str(out), "30", "48", "20", "8", "2"], capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, TSAN_OPTIONS="halt_on_error=1"))
    assert r.returncode == 0 and "WARNING: ThreadSanitizer" not in r.stderr, r.stderr[-3000:]
    assert r.stdout.strip() == "ok 30 frames"
