"""The dycore_test driver (the reference's program, src/dycore_test.F90,
over the C ABI) on the reference's mountain namelist."""
import subprocess
from pathlib import Path

import pytest

import gdc

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def driver():
    build = __import__("build")
    return build.OUT / "dycore_test"


def diag_lines(stdout):
    rows = []
    for line in stdout.splitlines():
        if line.startswith(" => "):
            f = line.split()
            rows.append(tuple(float(f[f.index(k) + 1]) for k in ("total_mass", "total_energy", "beta")))
    return rows


def test_driver_runs_the_namelist_like_the_model(native):
    out = subprocess.run([str(driver()), str(GOLDEN / "namelist.mountain"), "--steps", "6", "--log-every", "3"],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    rows = diag_lines(out.stdout)
    assert len(rows) == 3  # the initial state, then every 3 steps
    p, _, _ = gdc.read_namelist(GOLDEN / "namelist.mountain")
    m = gdc.Model(p)
    m.set_state(*gdc.ic_mountain_zonal_flow(p.num_lon, p.num_lat))
    m.run(6)
    assert m.diag() == rows[-1]  # printed with 17 significant digits: exact
    m.close()


def test_driver_refuses_an_unknown_test_case(native, tmp_path):
    nl = (GOLDEN / "namelist.mountain").read_text().replace("'mountain_zonal_flow'", "'no_such_case'", 1)
    path = tmp_path / "namelist.unknown"
    path.write_text(nl)
    out = subprocess.run([str(driver()), str(path), "--steps", "1"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 1 and "Unknown test case no_such_case" in out.stdout
