"""Run chosen kernels of the library on one small seeded case (for profilers).

    python -m minisod2d_gb300.profile_case --porder 7 --nx 12 --kernels convec,convec_mixed
    ncu ... python -m minisod2d_gb300.profile_case ...

Builds a structured mesh (``--nx``^3 hexes, ``--jitter``) with seeded fields
(``--kind`` 0 smooth, 1 shock-like), then runs each selected kernel
``--warmup`` + ``--iters`` times in order.  Kernels: convec, diffu,
convec_diffu (both residuals in one call, msod_convec_diffusion_ijk), convec_mixed, diffu_mixed (``--precision`` fp16 / bf16), estimator (plain
entropy viscosity), learned (features with the network + fallback, with a
freshly initialised network unless ``--weights`` names a weight file),
diffu_learned (the same followed by the per-element-viscosity diffusion;
needs ``--weights``),
diffu_nu (the diffusion with one viscosity per element),
tet_convec / tet_diffu (fem_convec / fem_diffu on the reference driver's
disconnected tetrahedra over the case's nodes).
"""
import argparse

from . import workload


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--porder", type=int, default=4)
    ap.add_argument("--nx", type=int, default=16)
    ap.add_argument("--jitter", type=float, default=0.05)
    ap.add_argument("--kind", type=int, default=0)
    ap.add_argument("--nmodes", type=int, default=8)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--kernels", default="convec,diffu")
    ap.add_argument("--precision", default="fp16", choices=["fp16", "bf16"])
    ap.add_argument("--weights", default=None)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--iters", type=int, default=1)
    a = ap.parse_args(argv)

    import torch

    from . import learn

    cfg = workload.Config("profile", a.porder, a.nx, a.jitter, a.kind, a.nmodes, a.seed)
    dev = workload.DeviceCase(workload.HostCase(cfg))
    out64 = None
    mlp = None
    tet = None
    calls = []
    for k in a.kernels.split(","):
        if k == "convec":
            calls.append(lambda: dev.convec())
        elif k == "diffu":
            calls.append(lambda: dev.diffu())
        elif k == "convec_diffu":
            calls.append(lambda: dev.convec_diffu())
        elif k in ("convec_mixed", "diffu_mixed"):
            if out64 is None:
                out64 = tuple(torch.empty(n * dev.npoin, dtype=torch.float64, device=dev.He.device)
                              for n in (1, 3, 1))
            fn = dev.convec_mixed if k == "convec_mixed" else dev.diffu_mixed
            calls.append(lambda fn=fn: fn(a.precision, out=out64))
        elif k in ("tet_convec", "tet_diffu"):
            if tet is None:
                tet = workload.TetCase(dev.host)
            calls.append(tet.convec if k == "tet_convec" else tet.diffu)
        elif k == "estimator":
            calls.append(lambda: learn.entropy_viscosity(dev))
        elif k in ("learned", "diffu_learned"):
            if mlp is None:
                mlp = learn.Mlp()
                if a.weights:
                    mlp.load(a.weights)
            if k == "learned":
                calls.append(lambda: learn.learned_viscosity(mlp, dev))
            else:
                calls.append(lambda: learn.diffusion_learned(mlp, dev))
        elif k == "diffu_nu":
            import torch as _t

            nu_c = _t.full((dev.nelem,), 1e-3, device=dev.rho.device)
            calls.append(lambda: learn.diffusion_ijk_nu(dev, nu_c))
        else:
            raise SystemExit("unknown kernel %r" % k)
    for fn in calls:
        for _ in range(a.warmup + a.iters):
            fn()
    torch.cuda.synchronize()
    print("ok: %s, porder %d, %d^3 hexes" % (a.kernels, a.porder, a.nx))


if __name__ == "__main__":
    main()
