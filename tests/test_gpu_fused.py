"""GPU checks of the one-call convection + diffusion (msod_convec_diffusion_ijk).

The call returns what msod_convec_ijk followed by msod_diffusion_ijk return on the same inputs
(main.f90:447,477 make the two calls back to back).  At porder 4 one kernel computes both from
one gather per element group with the same line-pass code as the two kernels; only the order of
the atomic additions into shared nodes differs, so the two forms agree to rounding: relative L2
<= 2e-6 per residual.  Other porders run the two kernels on one set of tables.  The fused results
are also held to the oracle criterion of the plain kernels (test_gpu_parity).
"""
import numpy as np
import pytest

from minisod2d_gb300 import capi, kernels
from oracle import oracle as O
from tests import refimpl
from tests.test_gpu_parity import TOL32, _case, _compare, _geom64, _geom_host, _oracle_convec, _oracle_diffu

pytestmark = pytest.mark.gpu

TOL_SAME = 2e-6


def _separate(dev):
    c = [x.clone() for x in dev.convec()]
    d = [x.clone() for x in dev.diffu()]
    return c, d


def _fused(dev):
    c, d = dev.convec_diffu()
    return [x.clone() for x in c], [x.clone() for x in d]


def _agree(a, b, label):
    errs = [refimpl.rel_l2(x.cpu().numpy(), y.cpu().numpy()) for x, y in zip(a, b)]
    print("FUSED %s mass %.2e mom %.2e ener %.2e" % (label, *errs))
    for name, e in zip(("mass", "mom", "ener"), errs):
        assert e <= TOL_SAME, (label, name, e)


@pytest.mark.parametrize("P,nx", [(4, 3), (5, 3), (7, 2), (2, 3), (3, 3), (6, 2)])
def test_fused_equals_separate_calls(cuda, P, nx):
    """nelem = nx^3 is not a multiple of the group size at any porder: the last group is partial."""
    host, dev = _case(cuda, P, nx, jitter=0.05, mu=1e-3)
    (cs, ds), (cf, df) = _separate(dev), _fused(dev)
    _agree(cf, cs, "P=%d convection" % P)
    _agree(df, ds, "P=%d diffusion" % P)


def test_fused_persistent_groups(cuda):
    """16^3 hexes at porder 4: 820 groups of five elements, more than the resident blocks, so the
    blocks loop over groups (the next group's ids and fields load between groups)."""
    host, dev = _case(cuda, 4, 16, jitter=0.05, mu=1e-3)
    (cs, ds), (cf, df) = _separate(dev), _fused(dev)
    _agree(cf, cs, "16^3 convection")
    _agree(df, ds, "16^3 diffusion")


@pytest.mark.parametrize("P,nx", [(4, 4), (7, 2)])
def test_fused_against_oracle(cuda, P, nx):
    host, dev = _case(cuda, P, nx, jitter=0.05, mu=1e-3)
    cf, df = _fused(dev)
    geom = _geom_host(dev)
    geom["P"] = P
    _compare(cf, _oracle_convec(host, geom), TOL32, "fused convec P=%d" % P, _oracle_convec(host, geom, np.float64))
    _compare(df, _oracle_diffu(host, geom), TOL32, "fused diffu P=%d" % P, _oracle_diffu(host, geom, np.float64))


def test_fused_reference_driver_case(cuda):
    """The reference driver's disconnected mesh (main.f90:320-413; no shared nodes, so the
    diffusion stage takes the plain line order): the fused call against the oracle."""
    import torch

    P, ne = 4, 7
    t = O.element_tables(P)
    connec, coord = O.create_mesh_disconnected(P, ne, t["xgp"])
    npn = ne * t["n"]
    He, gp = O.elem_jacobian(P, ne, npn, connec, coord, t["dNgp"], t["wgp"])
    f = O.reference_ic(P, ne, npn, connec)
    geom = dict(t, connec=connec, He=He, gpvol=gp)
    d = {k: torch.from_numpy(v).to(cuda) for k, v in dict(geom, **f).items() if isinstance(v, np.ndarray)}
    out = [torch.empty(n, device=cuda) for n in (npn, 3 * npn, npn, npn, 3 * npn, npn)]
    geo = (ne, npn, d["connec"], None, None, d["He"], d["gpvol"], d["dlxigp_ip"], None, d["invAtoIJK"], d["AtoI"],
           d["AtoJ"], d["AtoK"])
    kernels.full_convec_diffusion_ijk(*geo, 1.0, 1.0, d["u"], d["q"], d["rho"], d["pr"], d["E"], d["Tem"],
                                      d["mu_fluid"], d["mu_e"], d["mu_sgs"], *out)
    g64 = _geom64(dict(geom, P=P))
    rc = O.full_convec_ijk(P, ne, npn, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"])
    rc64 = O.full_convec_ijk(P, ne, npn, g64, f["u"], f["q"], f["rho"], f["pr"], f["E"], np.float64)
    _compare(out[:3], rc, TOL32, "fused convec reference-driver case", rc64)
    args = (f["rho"], f["u"], f["Tem"], f["mu_fluid"], f["mu_e"], f["mu_sgs"])
    rd = O.full_diffusion_ijk(P, ne, npn, geom, 1.0, 1.0, *args)
    rd64 = O.full_diffusion_ijk(P, ne, npn, g64, 1.0, 1.0, *args, np.float64)
    _compare(out[3:], rd, TOL32, "fused diffu reference-driver case", rd64)


def test_fused_outputs_are_intent_out(cuda):
    host, dev = _case(cuda, 4, 2, mu=1e-3)
    ref = _fused(dev)
    for x in (dev.Rmass, dev.Rmom, dev.Rener, dev.Dmass, dev.Dmom, dev.Dener):
        x.fill_(123.0)
    got = _fused(dev)
    for a, b in zip(ref[0] + ref[1], got[0] + got[1]):
        assert refimpl.rel_l2(a.cpu().numpy(), b.cpu().numpy()) <= TOL_SAME


def test_fused_rejects_bad_arguments(cuda):
    host, dev = _case(cuda, 4, 2)
    geo = dev.geometry()
    f = (dev.u, dev.q, dev.rho, dev.pr, dev.E, dev.Tem, dev.mu_fluid, dev.mu_e, dev.mu_sgs)
    with pytest.raises(capi.MsodError) as ei:  # the diffusion writes into the convection's arrays
        kernels.full_convec_diffusion_ijk(*geo, 1004.5, 0.71, *f, dev.Rmass, dev.Rmom, dev.Rener, dev.Rmass,
                                          dev.Dmom, dev.Dener)
    assert ei.value.code == capi.MSOD_ERR_INVALID_ARG
    with pytest.raises(capi.MsodError) as ei:
        kernels.full_convec_diffusion_ijk(*geo, 1004.5, 0.0, *f, dev.Rmass, dev.Rmom, dev.Rener, dev.Dmass,
                                          dev.Dmom, dev.Dener)
    assert ei.value.code == capi.MSOD_ERR_INVALID_ARG


def test_fused_follows_the_mode(cuda):
    """While msod_set_mode selects the FP16 tensor-core kernels the call makes the two drop-in
    calls, so it returns what they return in that mode."""
    host, dev = _case(cuda, 4, 3, mu=1e-3)
    kernels.set_mode("fp16")
    try:
        (cs, ds), (cf, df) = _separate(dev), _fused(dev)
    finally:
        kernels.set_mode("fp32")
    _agree(cf, cs, "fp16 mode convection")
    _agree(df, ds, "fp16 mode diffusion")
    plain = _fused(dev)
    assert refimpl.rel_l2(plain[1][2].cpu().numpy(), df[2].cpu().numpy()) > 0.0
