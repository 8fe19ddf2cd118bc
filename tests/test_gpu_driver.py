"""The driver program (nekbone_gb300/bin/nekbone, driver.f over the C ABI)
on the C1 configuration, against the reference's own Fortran run of it
(tests/golden/fortran_c1_4x4x4_lx10.npz): the printed cg lines of the timed
call to 1e-10 relative (the GPU's fused multiply-adds and tree reductions
against the reference's sequential sums), the flop counts exactly."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
DRIVER = ROOT / "nekbone_gb300" / "bin" / "nekbone"
GOLDEN = Path(__file__).parent / "golden" / "fortran_c1_4x4x4_lx10.npz"


def _run(tmp_path, rea, *flags):
    (tmp_path / "data.rea").write_text(rea)
    if not DRIVER.exists():
        import nekbone_gb300  # noqa: F401  (the library exists; build the driver)
        import importlib.util
        spec = importlib.util.spec_from_file_location("nbbuild", ROOT / "nekbone_gb300" / "build.py")
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        m.build_driver()
    p = subprocess.run([str(DRIVER), *flags], cwd=tmp_path, capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr
    return p.stdout


def test_driver_c1_matches_reference(tmp_path):
    if not GOLDEN.exists():
        pytest.skip("C1 fixture not generated")
    g = np.load(GOLDEN)
    out = _run(tmp_path, ".true.    = ifbrick\n64 64 1 = iel0,ielN,stride\n"
                         "10 10 1 = nx0,nxN,stride\n0 0 0 = npx,npy,npz\n0 0 0 = mx,my,mz\n",
               "--digits")
    cg = [l.split()[1:] for l in out.splitlines() if l.startswith("cg:")]
    assert len(cg) == 4                       # two calls, two lines each
    it0, final = cg[2], cg[3]                 # the timed call
    log = g["log_timed"]
    rtz1, pap, rtr = log[1::3], log[2::3], log[3::3]
    ref_final = [np.sqrt(rtr[-1]), rtz1[-1] / pap[-1], rtz1[-1] / rtz1[-2], pap[-1]]
    assert int(it0[0]) == 0 and int(final[0]) == 101
    assert abs(float(it0[1]) - np.sqrt(log[0])) <= 1e-10 * np.sqrt(log[0])
    for got, ref in zip(final[1:], ref_final):
        assert abs(float(got) - ref) <= 1e-10 * abs(ref), (got, ref)
    m = re.search(r"Setup Flop =\s*(\S+), Solver Flop =\s*(\S+)", out)
    assert float(m.group(1)) == 100 * (19 * 1000 + 12 * 10 * 1000) * 64
    assert float(m.group(2)) == 101 * 15 * 64000
    assert "Avg MFlops" in out


def test_driver_element_and_order_ranges(tmp_path):
    out = _run(tmp_path, ".false.\n2 6 2\n4 6 2\n0 0 0\n0 0 0\n")
    runs = re.findall(r"nelt =\s*(\d+), np =\s*1, nx1 =\s*(\d+)", out)
    assert runs == [("2", "4"), ("4", "4"), ("6", "4"), ("2", "6"), ("4", "6"), ("6", "6")]


def test_driver_rejects_bad_ranges(tmp_path):
    out = _run(tmp_path, ".true.\n8 4 1\n6 6 1\n0 0 0\n0 0 0\n")
    assert "iel0 > ielN" in out
