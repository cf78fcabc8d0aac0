"""The bounds-checking build of the library (device-side bounds checks
reported as a status word, pfs_bounds_status): every entry point of the
timestep, on grids from 2x1 to 1000x130, leaves the record empty, and the
drop-in results still equal the reference's golden vectors.

A checked access that falls outside its buffer is skipped, never performed, so
these runs cannot fault the GPU whatever the indices. The GPU test builds the
bounds library in-tree (libpfs_gb300_bounds.so) and runs tests/bounds_cases.py
against it in a subprocess (PFS_LIBRARY selects the library)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_normal_build_has_no_bounds_record(pfs_lib):
    """The normal build answers unsupported (no device work; runs without a GPU)."""
    with pytest.raises(pfs_lib.PFSError) as e:
        pfs_lib.bounds_status()
    assert e.value.status == 4  # PFS_ERR_UNSUPPORTED


@pytest.mark.gpu
def test_bounds_build_records_no_access_outside_its_buffer(cuda_device):
    from probabilistic_fluid_simulation_gb300 import build
    lib = build.build(bounds=True)
    env = dict(os.environ, PFS_LIBRARY=lib)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "bounds_cases.py")], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stderr[-3000:]
    recs = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
    kinds = {rec["case"].split()[0] for rec in recs}
    assert {"dropin", "session", "precision", "sweeps", "ensemble"} <= kinds, kinds
    bad = [rec for rec in recs if rec["count"] != 0]
    assert not bad, bad[:5]
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from golden_util import cases
    golden = [rec for rec in recs if rec["case"].startswith("dropin") and "equal" in rec]
    assert len(golden) == len(cases()) and all(rec["equal"] for rec in golden)
    # the sweep entry points ran (only sizes an entry point does not take are rejected, on the host)
    assert all(not rec.get("rejected") for rec in recs if rec["case"].startswith("sweeps")), recs
