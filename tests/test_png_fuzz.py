"""The command-line driver's PNG codec under AddressSanitizer and
UndefinedBehaviorSanitizer (host only). Decoder: seeds of every colour type,
bit depth and both interlace methods, each mutated thousands of times; every
mutated file decodes to an image of its stated size or is rejected with a
message, with no memory error. Encoder: round trips of images of many sizes
and kinds of content."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import png_util as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "probabilistic_fluid_simulation_gb300", "cli")
SRC = os.path.join(ROOT, "tests", "cpp", "png_fuzz_main.cpp")


def seeds(d):
    rng = np.random.default_rng(11)
    files = []
    cases = [(6, 8, False), (6, 8, True), (2, 8, False), (0, 1, True), (0, 4, False), (4, 8, True), (3, 2, False),
             (3, 8, True)]
    for k, (ct, depth, interlace) in enumerate(cases):
        w, h = 13 + k, 9 + 2 * k
        if ct == 3:
            samples = rng.integers(0, 1 << depth, (h, w)).astype(np.uint8)
            pal = rng.integers(0, 256, (1 << depth, 3)).astype(np.uint8)
            data = P.encode(samples, ct, depth, interlace, palette=pal, trns=[0, 128])
        else:
            chans = {0: 1, 2: 3, 4: 2, 6: 4}[ct]
            shape = (h, w) if chans == 1 else (h, w, chans)
            data = P.encode(rng.integers(0, 1 << depth, shape).astype(np.uint8), ct, depth, interlace)
        path = os.path.join(d, f"seed{k}.png")
        with open(path, "wb") as f:
            f.write(data)
        files.append(path)
    return files


def test_decoder_survives_mutations(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host compiler")
    exe = str(tmp_path / "png_fuzz")
    cmd = [gxx, "-O1", "-g", "-std=c++17", "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-I", CLI,
           SRC, os.path.join(CLI, "png.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("sanitizers not available")
    assert r.returncode == 0, r.stderr
    files = seeds(str(tmp_path))
    r = subprocess.run([exe, "1500", "7"] + files, capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1"))
    assert r.returncode == 0, r.stderr[-3000:]
    decoded, rejected = (int(x) for x in r.stdout.split()[1::2])
    assert decoded + rejected == 1500 * len(files) and rejected > 0


def test_encoder_round_trips_under_sanitizers(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host compiler")
    exe = str(tmp_path / "png_encode_asan")
    src = os.path.join(ROOT, "tests", "cpp", "png_encode_asan_main.cpp")
    cmd = [gxx, "-O1", "-g", "-std=c++17", "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-I", CLI,
           src, os.path.join(CLI, "png.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("sanitizers not available")
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "400", "5"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert r.stdout.strip() == "ok 400"
