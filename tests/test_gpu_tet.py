"""GPU parity of the linear-tetrahedron kernels (fem_convec, fem_diffu,
tet_jacobian) through the C ABI against the oracle.

Criteria: tet_jacobian bit for bit (FP32 and FP64, the same rounding as
the oracle); FP64 kernels within 1e-12 of the FP64 oracle; FP32 kernels
within max(1e-5, 4 x the oracle's own FP32 floor) of the FP64 oracle (the
GPU contracts multiply-adds, the reference's FP32 build does not).  Both the
driver's disconnected mesh (vector reductions) and a shared-node mesh (scalar
reductions that collide) are covered.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import refimpl as R

pytestmark = pytest.mark.gpu


def _fields(npoin, nelem, seed=0):
    rng = np.random.default_rng(seed)
    f = dict(rho=1 + rng.random(npoin), pr=1 + rng.random(npoin), E=2 + rng.random(npoin),
             u=rng.standard_normal(3 * npoin), Tem=1 + rng.random(npoin), mu_fluid=0.1 * rng.random(npoin),
             mu_e=0.1 * rng.random(4 * nelem), mu_sgs=0.1 * rng.random(4 * nelem))
    f["q"] = (f["u"].reshape(3, -1) * f["rho"]).reshape(-1)
    return {k: v.astype(np.float32) for k, v in f.items()}


class TetCase:
    def __init__(self, cuda, kind, dtype, seed=0):
        import torch

        from minisod2d_gb300 import fem, kernels

        self.torch_dtype = torch.float32 if dtype == np.float32 else torch.float64
        if kind == "driver":
            self.nelem = 1000
            connec, coord, self.npoin = fem.tet_mesh_disconnected(self.nelem)
        else:
            connec, coord, self.nelem, self.npoin = R.tet_mesh_shared(6, 0.2, seed)
        self.connec_h, self.coord_h = connec, coord.astype(dtype)
        self.t = fem.tet_element_tables(dtype)
        dev = lambda a, dt=self.torch_dtype: torch.as_tensor(np.ascontiguousarray(a), device=cuda).to(dt)
        self.dev = dev
        self.connec = dev(connec, torch.int32)
        self.coord = dev(self.coord_h)
        self.Ngp, self.dNgp, self.wgp = dev(self.t["Ngp"]), dev(self.t["dNgp"]), dev(self.t["wgp"])
        self.He = torch.empty(36 * self.nelem, dtype=self.torch_dtype, device=cuda)
        self.gpvol = torch.empty(4 * self.nelem, dtype=self.torch_dtype, device=cuda)
        kernels.tet_jacobian(self.nelem, self.npoin, self.connec, self.coord, self.dNgp, self.wgp, self.gpvol, self.He)
        self.f_h = {k: v.astype(dtype) for k, v in _fields(self.npoin, self.nelem, seed + 1).items()}
        self.f = {k: dev(v) for k, v in self.f_h.items()}
        self.cuda = cuda

    def outputs(self, fill=0.0):
        import torch

        return tuple(torch.full((n * self.npoin,), fill, dtype=self.torch_dtype, device=self.cuda) for n in (1, 3, 1))

    def convec(self, He=None, out=None):
        from minisod2d_gb300 import kernels

        out = out or self.outputs()
        f = self.f
        kernels.fem_convec(self.nelem, self.npoin, self.connec, self.Ngp, self.dNgp, self.He if He is None else He,
                           self.gpvol, f["u"], f["q"], f["rho"], f["pr"], f["E"], *out)
        return out

    def diffu(self, out=None):
        from minisod2d_gb300 import kernels

        out = out or self.outputs()
        f = self.f
        kernels.fem_diffu(self.nelem, self.npoin, self.connec, self.Ngp, self.dNgp, self.He, self.gpvol, 1.0, 0.71,
                          f["rho"], f["u"], f["Tem"], f["mu_fluid"], f["mu_e"], f["mu_sgs"], *out)
        return out

    def geometry_host(self):
        return self.He.cpu().numpy(), self.gpvol.cpu().numpy()

    def oracle(self, which, dtype):
        He, gp = self.geometry_host()
        f, t = self.f_h, self.t
        if which == "convec":
            return O.fem_convec(self.nelem, self.npoin, self.connec_h, t["Ngp"], t["dNgp"], He, gp, f["u"], f["q"],
                                f["rho"], f["pr"], f["E"], dtype, nthreads=8)
        return O.fem_diffu(self.nelem, self.npoin, self.connec_h, t["Ngp"], t["dNgp"], He, gp, 1.0, 0.71, f["rho"],
                           f["u"], f["Tem"], f["mu_fluid"], f["mu_e"], f["mu_sgs"], dtype, nthreads=8)


def _errs(gpu, ref):
    return [R.rel_l2(g.cpu().numpy().astype(np.float64), r.astype(np.float64)) for g, r in zip(gpu, ref)]


@pytest.mark.parametrize("kind", ["driver", "shared"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_tet_jacobian_bit_exact(cuda, kind, dtype):
    c = TetCase(cuda, kind, dtype)
    He, gp = O.tet_jacobian(c.nelem, c.npoin, c.connec_h, c.coord_h, c.t["dNgp"], c.t["wgp"], dtype)
    g_He, g_gp = c.geometry_host()
    assert np.array_equal(g_He, He) and np.array_equal(g_gp, gp)


@pytest.mark.parametrize("kind", ["driver", "shared"])
@pytest.mark.parametrize("which", ["convec", "diffu"])
def test_tet_fp32_parity(cuda, kind, which):
    c = TetCase(cuda, kind, np.float32)
    gpu = c.convec() if which == "convec" else c.diffu()
    ref64 = c.oracle(which, np.float64)
    floor = _errs([__import__("torch").as_tensor(x) for x in c.oracle(which, np.float32)], ref64)
    errs = _errs(gpu, ref64)
    print("TET %s %s err=%s floor32=%s" % (which, kind, ["%.2e" % e for e in errs], ["%.2e" % e for e in floor]))
    for e, fl in zip(errs, floor):
        assert e <= max(1e-5, 4.0 * fl), (e, fl)


@pytest.mark.parametrize("kind", ["driver", "shared"])
@pytest.mark.parametrize("which", ["convec", "diffu"])
def test_tet_fp64_parity(cuda, kind, which):
    c = TetCase(cuda, kind, np.float64)
    gpu = c.convec() if which == "convec" else c.diffu()
    for e in _errs(gpu, c.oracle(which, np.float64)):
        assert e < 1e-12


def test_tet_vector_and_scalar_paths_agree(cuda):
    """The driver's mesh with aligned arrays takes the 16-byte loads and the
    vector reductions; misaligned views take the scalar forms.  No node is
    shared, so every node receives one addition and the results are equal."""
    import torch

    c = TetCase(cuda, "driver", np.float32)
    a = c.convec()
    big = torch.empty(36 * c.nelem + 1, dtype=torch.float32, device=cuda)
    big[1:] = c.He
    He_mis = big[1:]                                   # 4-byte offset: no vector loads
    outs = tuple(torch.zeros(n * c.npoin + 1, dtype=torch.float32, device=cuda)[1:] for n in (1, 3, 1))
    b = c.convec(He=He_mis, out=outs)                  # misaligned outputs: scalar reductions
    for x, y in zip(a, b):
        assert torch.equal(x, y)


def test_tet_outputs_are_intent_out(cuda):
    import torch

    c = TetCase(cuda, "shared", np.float32)
    a = c.diffu()
    b = c.diffu(out=c.outputs(fill=123.0))
    for x, y in zip(a, b):
        assert R.rel_l2(x.cpu().numpy(), y.cpu().numpy()) < 1e-6
        assert float(torch.abs(y).max()) < 1e3


def test_tet_rejects_bad_arguments(cuda):
    import torch

    from minisod2d_gb300 import capi, kernels

    c = TetCase(cuda, "driver", np.float32)
    out = c.outputs()
    with pytest.raises(ValueError):  # wrong table size
        kernels.fem_convec(c.nelem, c.npoin, c.connec, c.Ngp[:8], c.dNgp, c.He, c.gpvol, c.f["u"], c.f["q"],
                           c.f["rho"], c.f["pr"], c.f["E"], *out)
    with pytest.raises(capi.MsodError) as ei:
        capi.call("msod_fem_diffu", c.nelem, c.npoin, c.connec.data_ptr(), c.Ngp.data_ptr(), c.dNgp.data_ptr(),
                  c.He.data_ptr(), c.gpvol.data_ptr(), 1.0, 0.0, *[c.f[k].data_ptr() for k in
                  ("rho", "u", "Tem", "mu_fluid", "mu_e", "mu_sgs")], *[t.data_ptr() for t in out],
                  torch.cuda.current_stream().cuda_stream)
    assert ei.value.code == capi.MSOD_ERR_INVALID_ARG  # Pr = 0
    bad = c.connec.clone()
    bad[5] = c.npoin + 7
    kernels.set_checked(True)
    try:
        with pytest.raises(capi.MsodError) as ei:
            kernels.fem_convec(c.nelem, c.npoin, bad, c.Ngp, c.dNgp, c.He, c.gpvol, c.f["u"], c.f["q"], c.f["rho"],
                               c.f["pr"], c.f["E"], *out)
        assert ei.value.code == capi.MSOD_ERR_BAD_TABLES
    finally:
        kernels.set_checked(False)
    # unchecked: the bad entry is clamped for reading and skipped in the assembly
    kernels.fem_convec(c.nelem, c.npoin, bad, c.Ngp, c.dNgp, c.He, c.gpvol, c.f["u"], c.f["q"], c.f["rho"],
                       c.f["pr"], c.f["E"], *out)
    torch.cuda.synchronize()
