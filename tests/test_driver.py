"""The benchmark driver (msod_driver, main.f90 on the C ABI) and the reference
driver's own case (create_mesh, the initial condition of main.f90:320-361).

CPU: the timers.dat / results_*.dat line formats (main.f90:499-500, :586-599)
and the library's mesh and initial condition against the oracle, bit for bit.
GPU: a small run of the driver: timers.dat, the results files against the
FP64 oracle, the JSON summary.
"""
import json
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests import refimpl as R

HERE = os.path.dirname(os.path.abspath(__file__))
DRIVER = os.path.join(os.path.dirname(HERE), "minisod2d_gb300", "msod_driver")


def _driver():
    from minisod2d_gb300 import build

    build.build()
    return DRIVER


def test_driver_line_formats():
    out = subprocess.run([_driver(), "--format-check"], capture_output=True, text=True, check=True).stdout
    lines = out.splitlines()
    # (i3,1x,4(f16.8,1x)): 3 + 4 x 17 columns, a blank after every value
    assert lines[0] == "  7       0.00010690      12.50000000       0.00000000  123456.78901234 "
    assert lines[1].startswith("*** ") and len(lines[1]) == 3 + 1 + 4 * 17
    assert lines[2] == "1.0690000000000000E-004"
    assert lines[3] == ("          42   1.00000000E+00  -2.49999994E-03   0.00000000E+00   3.00000000E+07"
                        "  -1.00000000E+00")


def test_driver_rejects_bad_options():
    r = subprocess.run([_driver(), "--mesh", "spiral"], capture_output=True, text=True)
    assert r.returncode == 2
    r = subprocess.run([_driver(), "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2


@pytest.mark.parametrize("P", [2, 4])
def test_reference_case_equals_the_oracle(P):
    from minisod2d_gb300 import fem

    t, ot = fem.element_tables(P), O.element_tables(P)
    c, x, npoin = fem.mesh_disconnected(P, 11, t)
    oc, ox = O.create_mesh_disconnected(P, 11, ot["xgp"])
    assert np.array_equal(c, oc) and np.array_equal(x, ox)
    f, of = fem.reference_ic(P, 11, npoin, c), O.reference_ic(P, 11, npoin, oc)
    for k in f:
        assert np.array_equal(f[k], of[k]), k


@pytest.mark.gpu
def test_driver_run_matches_the_oracle(cuda, tmp_path):
    P, nelem, nruns = 4, 96, 3
    r = subprocess.run([_driver(), "--porder", str(P), "--nelem", str(nelem), "--nruns", str(nruns), "--debug",
                        "--out", str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Avg. convective time" in r.stdout and "Basic TET results:" in r.stdout
    rows = (tmp_path / "timers.dat").read_text().splitlines()
    assert len(rows) == nruns
    pat = re.compile(r"^[ \d]{3}( [ \d.]{15}\d){4} $")
    assert all(pat.match(row) for row in rows), rows
    assert all(float(v) > 0 for row in rows for v in row.split()[1:])
    summary = json.loads((tmp_path / "results.json").read_text())
    n = (P + 1) ** 3
    assert summary["nelem"] == nelem and summary["npoin"] == nelem * n and summary["npoin_tet"] == nelem * n

    # The results files against the FP64 oracle on the same case.
    t = O.element_tables(P)
    connec, coord = O.create_mesh_disconnected(P, nelem, t["xgp"])
    npoin = nelem * n
    f = O.reference_ic(P, nelem, npoin, connec)
    He, gp = O.elem_jacobian(P, nelem, npoin, connec, coord, t["dNgp"], t["wgp"])
    geom = dict(t, connec=connec, He=He, gpvol=gp)
    ref_c = O.full_convec_ijk(P, nelem, npoin, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], dtype=np.float64,
                              nthreads=8)
    ref_d = O.full_diffusion_ijk(P, nelem, npoin, geom, 1.0, 1.0, f["rho"], f["u"], f["Tem"], f["mu_fluid"],
                                 f["mu_e"], f["mu_sgs"], dtype=np.float64, nthreads=8)
    for name, ref in (("results_convec.dat", ref_c), ("results_diffu.dat", ref_d)):
        a = np.loadtxt(tmp_path / name)
        assert a.shape == (npoin, 6) and np.array_equal(a[:, 0], np.arange(1, npoin + 1))
        got = (a[:, 1], np.concatenate([a[:, 2], a[:, 3], a[:, 4]]), a[:, 5])
        for g, r64 in zip(got, ref):
            assert R.rel_l2(g, r64) < 1e-5, name


@pytest.mark.gpu
def test_driver_structured_mesh_matches_the_oracle(cuda, tmp_path):
    """--mesh structured --fields smooth: the scaled shared-node workload through the driver."""
    from minisod2d_gb300 import fem

    P, nx = 2, 3
    r = subprocess.run([_driver(), "--porder", str(P), "--mesh", "structured", "--nx", str(nx), "--jitter", "0.05",
                        "--fields", "smooth", "--seed", "3", "--nruns", "2", "--debug", "--out", str(tmp_path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    t = fem.element_tables(P)
    connec, coord, nelem, npoin = fem.structured_mesh(P, nx, nx, nx, t, 0.05, 3)
    f = fem.fields_recipe(0, 8, 3, npoin, coord)
    n = (P + 1) ** 3
    ot = O.element_tables(P)
    He, gp = O.elem_jacobian(P, nelem, npoin, connec, coord, ot["dNgp"], ot["wgp"])
    geom = dict(ot, connec=connec, He=He, gpvol=gp)
    ones = np.ones(nelem * n, np.float32)
    ref_c = O.full_convec_ijk(P, nelem, npoin, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], dtype=np.float64)
    ref_d = O.full_diffusion_ijk(P, nelem, npoin, geom, 1.0, 1.0, f["rho"], f["u"], f["Tem"], f["mu_fluid"], ones,
                                 ones, dtype=np.float64)
    for name, ref in (("results_convec.dat", ref_c), ("results_diffu.dat", ref_d)):
        a = np.loadtxt(tmp_path / name)
        got = (a[:, 1], np.concatenate([a[:, 2], a[:, 3], a[:, 4]]), a[:, 5])
        for g, r64 in zip(got, ref):
            assert R.rel_l2(g, r64) < 2e-5, name


@pytest.mark.gpu
@pytest.mark.parametrize("precision,mu_e,conv_bound,diff_bound", [
    ("fp32", "given", 1e-5, 1e-4), ("fp16", "given", 2e-4, 5e-3), ("bf16", "given", 1e-3, 2e-2),
    ("fp32", "plain", 1e-5, 1e-4), ("fp32", "learned", 1e-5, 1.0), ("fp16", "learned", 2e-4, 1.0)])
def test_driver_modes(cuda, tmp_path, precision, mu_e, conv_bound, diff_bound):
    """The driver's switches (main.f90's timing loop with the precision and viscosity forms of
    msod_set_mode): every mode runs, keeps the timers.dat format, times each call with CUDA events
    beside the wall clock, and its FP64 check (the FP64 build on the same inputs; for an estimated
    viscosity, with the plain estimator's mu_e) stays within the mode's accuracy."""
    from minisod2d_gb300 import learn

    nruns = 2
    args = [_driver(), "--porder", "4", "--mesh", "structured", "--nx", "6", "--jitter", "0.05", "--fields", "shock",
            "--seed", "3", "--nruns", str(nruns), "--precision", precision, "--mu-e", mu_e, "--fp64-check",
            "--out", str(tmp_path)]
    if mu_e == "learned":
        args += ["--weights", learn.shipped_weights("learned_48")]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Avg. convective time" in r.stdout and "FP64 check" in r.stdout
    pat = re.compile(r"^[ \d]{3}( [ \d.]{15}\d){4} $")
    for name in ("timers.dat", "timers_events.dat"):
        rows = (tmp_path / name).read_text().splitlines()
        assert len(rows) == nruns and all(pat.match(row) for row in rows), (name, rows)
    s = json.loads((tmp_path / "results.json").read_text())
    assert s["precision"] == precision and s["mu_e"] == mu_e and s["fp64_check"] is True
    assert all(v > 0 for v in s["avg_event_s"].values())
    assert all(s["avg_event_s"][k] <= s["avg_s"][k] * 1.5 + 1e-4 for k in s["avg_s"])
    f = json.loads((tmp_path / "fp64_check.json").read_text())
    print("DRIVER %s %s %s" % (precision, mu_e, {k: "%.2e" % v for k, v in f.items() if k not in ("precision", "mu_e")}))
    assert max(f["Rmass"], f["Rmom"], f["Rener"]) < conv_bound
    assert max(f["Dmom"], f["Dener"]) < min(diff_bound, 0.1)
    assert f["Dmass"] < diff_bound
