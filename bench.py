#!/usr/bin/env python
"""Throughput of the hex convection + diffusion residuals (one JSON line).

A step is one evaluation of both residuals -- full_convec_ijk then
full_diffusion_ijk -- over the plain_64 workload: 64^3 hexes, porder 4
(257^3 = 16,974,593 shared nodes), +-5% seeded vertex jitter, seeded Fourier
fields (FP32).  value = 5 * npoin / (time per step) in GDOF/s: one
degree of freedom per unique node and conserved variable (mass, 3 momentum,
energy) for the full right-hand side.  Inputs (2.4 GB per call) exceed the
129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N --steps K --warmup W]            this library on the GPU
  python bench.py --impl reference [--steps K --warmup W]    the reference algorithm on the host cores

Under torchrun each rank runs its own replica of the workload (weak scaling,
no collective on the data path); rank 0 prints the max-over-ranks timing.

On one GPU the line also carries "variants": the linear-tetrahedron kernels
on the reference driver's tet mesh over the plain_64 nodes, the
mixed-precision kernels on the 32^3 porder-7 workload, the learned viscosity
on a held-out seed of the 48^3 shock workload and the combined 96^3 porder-5
workload, each timed with CUDA events, with errors against the FP64 build of
the same kernels (--no-variants skips them).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "convec+diffu GDOF/s & % HBM roofline; mixed/learned vs plain at stated error"
FALLBACK_HBM_GBS = 6800.0


def algorithmic_bytes(nelem, n, npoin):
    """Compulsory bytes per call: every input read once, every output written once."""
    conv = nelem * n * (4 + 36 + 4) + npoin * (36 + 20)
    diff = nelem * n * (4 + 36 + 4 + 4 + 4) + npoin * (24 + 20)
    return conv, diff


def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            v = float(json.load(f)["hbm_gbs"])
        return v, "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        """Start sampling every 50 ms; returns once the first sample is in, so
        that the samples that follow fall inside the timed region."""
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 5.0 and os.path.getsize(self.file.name) == 0:
                time.sleep(0.01)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
        self.file.close()
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    return rank, local, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world, device):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_traffic(workload_name):
    """Per-launch DRAM bytes of each kernel from the committed ncu summary (or None)."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(workload_name)
    except Exception:
        return None


# --------------------------------------------------------------------------------------
# CPU legs: the oracle (restatement of the reference's CPU path) on a bounded sample
# --------------------------------------------------------------------------------------
def cpu_sample_case(cfg, host, nsample):
    """A contiguous slab of `nsample` elements from the middle of the mesh with its
    metric computed by the oracle's elem_jacobian."""
    from oracle import oracle as O

    n = cfg.nnode
    e0 = max(0, host.nelem // 2 - nsample // 2)
    e1 = min(host.nelem, e0 + nsample)
    con = np.ascontiguousarray(host.connec.reshape(n, host.nelem)[:, e0:e1]).reshape(-1)
    t = host.tables
    He, gp = O.elem_jacobian(cfg.porder, e1 - e0, host.npoin, con, host.coord, t["dNgp"], t["wgp"])
    geom = dict(t, connec=con, He=He, gpvol=gp)
    mu = np.zeros((e1 - e0) * n, np.float32)
    return geom, e1 - e0, mu


def cpu_step(cfg, host, geom, ne, mu, nthreads):
    from oracle import oracle as O

    f = host.fields
    O.full_convec_ijk(cfg.porder, ne, host.npoin, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"],
                      nthreads=nthreads)
    O.full_diffusion_ijk(cfg.porder, ne, host.npoin, geom, cfg.Cp, cfg.Pr, f["rho"], f["u"], f["Tem"],
                         f["mu_fluid"], mu, mu, nthreads=nthreads)


def calibrate_sample(cfg, host, nthreads, seconds):
    """Number of elements whose convec+diffu takes about `seconds` on `nthreads`
    (a warm-up call first, then a timed probe of about a tenth of the target)."""
    ne = 64 * nthreads
    geom, ne, mu = cpu_sample_case(cfg, host, ne)
    cpu_step(cfg, host, geom, ne, mu, nthreads)
    for _ in range(2):
        t0 = time.perf_counter()
        cpu_step(cfg, host, geom, ne, mu, nthreads)
        dt = max(time.perf_counter() - t0, 1e-4)
        if dt > 0.05 * seconds or ne >= host.nelem:
            break
        ne = min(host.nelem, int(ne * 0.1 * seconds / dt) + 1)
        geom, ne, mu = cpu_sample_case(cfg, host, ne)
    want = int(ne * seconds / dt)
    return max(64, min(host.nelem, want))


def cpu_baseline(cfg, host, seconds=15.0):
    """The serial oracle (the faithful single-core restatement) on a bounded sample
    of about `seconds` of CPU work."""
    ns = calibrate_sample(cfg, host, 1, seconds)
    geom, ne, mu = cpu_sample_case(cfg, host, ns)
    t0 = time.perf_counter()
    cpu_step(cfg, host, geom, ne, mu, 1)
    dt = time.perf_counter() - t0
    dofs = 5.0 * host.npoin * ne / host.nelem
    return {"value": dofs / dt / 1e9, "unit": "GDOF/s", "cores": 1, "kind": "port",
            "sample": "%d of %d elements (a contiguous slab), convec+diffu, serial oracle, %.1f s; DOFs "
                      "prorated by element share" % (ne, host.nelem, dt)}


def host_link(ups, downs, s_up, s_down, reps=3):
    """This box's pinned-host <-> device link, measured with the e2e step's own copies before its
    timed region: `ups` and `downs` are (device pointer, host pointer, bytes) triples, issued
    through msod_h2d / msod_d2h on two streams, uploads alone, downloads alone and both at once
    (as the pipelined step overlaps them).  Returns GB/s and ms per step's copies; both_ms is the
    least time of a step's copies, the floor of the e2e step."""
    import torch

    from minisod2d_gb300 import capi

    L = capi.lib()

    def timed(up, down):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s_up)
        s_down.wait_event(a)
        for _ in range(reps):
            if up:
                for d, h, n in ups:
                    capi.check(L.msod_h2d(d, h, n, s_up.cuda_stream))
            if down:
                for d, h, n in downs:
                    capi.check(L.msod_d2h(h, d, n, s_down.cuda_stream))
        s_up.wait_stream(s_down)
        b.record(s_up)
        b.synchronize()
        return a.elapsed_time(b) / reps

    timed(True, True)
    bu, bd = sum(n for _, _, n in ups), sum(n for _, _, n in downs)
    tu, td, tb = timed(True, False), timed(False, True), timed(True, True)
    return {"h2d_ms": tu, "d2h_ms": td, "both_ms": tb, "h2d_gbs": bu / tu / 1e6, "d2h_gbs": bd / td / 1e6,
            "both_gbs": (bu + bd) / tb / 1e6}


def workload_config(cfg, nelem, npoin):
    """The `config` of both arms' JSON lines: the workload alone (arm details sit outside it)."""
    Bc, Bd = algorithmic_bytes(nelem, cfg.nnode, npoin)
    return {"workload": cfg.name, "porder": cfg.porder, "nelem": nelem, "npoin": npoin, "jitter": cfg.jitter,
            "l2": "inputs %.2f GB per call > 129 MB L2, no flush" % ((Bc + Bd) / 2e9)}


class OracleHostCase:
    """The workload's host arrays built by the oracle alone -- element tables, structured mesh,
    seeded fields, bit for bit those of the library's setup (tests/test_oracle_kat.py) -- so that
    the reference arm loads no product code."""

    def __init__(self, cfg):
        from oracle import oracle as O

        self.cfg = cfg
        self.tables = O.element_tables(cfg.porder)
        self.connec, self.coord, self.nelem, self.npoin = O.structured_mesh(cfg.porder, cfg.nx, self.tables,
                                                                            cfg.jitter, cfg.seed)
        self.fields = O.fields_recipe(cfg.kind, cfg.nmodes, cfg.seed, self.npoin, self.coord)


def run_reference(args, cfg):
    """--impl reference: the reference algorithm (the oracle port) on all host cores."""
    from oracle import oracle as O

    O.lib()
    host = OracleHostCase(cfg)
    nth = O.cpu_count()
    per_step = max(1.0, min(5.0, 90.0 / max(1, args.steps + args.warmup)))
    ns = calibrate_sample(cfg, host, nth, per_step)
    geom, ne, mu = cpu_sample_case(cfg, host, ns)
    for _ in range(args.warmup):
        cpu_step(cfg, host, geom, ne, mu, nth)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_step(cfg, host, geom, ne, mu, nth)
    dt = (time.perf_counter() - t0) / max(1, args.steps)
    dofs = 5.0 * host.npoin * ne / host.nelem
    value = dofs / dt / 1e9
    sample = ("%d of %d elements per step (a contiguous slab), convec+diffu, OpenMP oracle on %d threads; DOFs "
              "prorated by element share" % (ne, host.nelem, nth))
    out = {"metric": METRIC, "value": value, "unit": "GDOF/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered structured mesh, Fourier fields)",
           "impl": "reference", "config": workload_config(cfg, host.nelem, host.npoin),
           "parallelism": "OpenMP element loop on %d host threads (rank 0 only)" % nth,
           "inputs": "built by the oracle (oracle/): no product library loaded",
           "cpu_baseline": {"value": value, "unit": "GDOF/s", "cores": nth, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "GDOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# --------------------------------------------------------------------------------------
# GPU leg
# --------------------------------------------------------------------------------------
def run_ours(args, cfg, rank, local, world):
    import ctypes as C

    import torch

    from minisod2d_gb300 import build, capi, workload

    build.build()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    capi.call("msod_init", local)
    host = workload.HostCase(cfg)
    dev = workload.DeviceCase(host, device=device)
    torch.cuda.synchronize()
    n = cfg.nnode
    Bc, Bd = algorithmic_bytes(dev.nelem, n, dev.npoin)
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        dev.convec()
        dev.diffu()
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        dev.convec()
        ev[k][1].record(stream)
        dev.diffu()
        ev[k][2].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    total_ms = t_start.elapsed_time(t_end)
    conv_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in ev]))
    diff_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in ev]))
    total_ms = max_over_ranks(total_ms, world, device)
    ms_step = total_ms / args.steps
    value = world * 5.0 * dev.npoin / (ms_step * 1e-3) / 1e9

    # e2e through the C ABI with host buffers: every step copies its nine input
    # fields from pinned host memory (msod_h2d), runs both residual calls and
    # copies its six residual arrays back (msod_d2h).  Steps are pipelined over
    # two device buffer sets and three streams: the uploads of step k+1 and the
    # downloads of step k-1 overlap the kernels of step k (the copy engines and
    # the SMs work at the same time); the timed region holds K whole steps,
    # pipeline fill and drain included.
    e2e = None
    if not args.no_e2e:
        L = capi.lib()
        ins = ("u", "q", "rho", "pr", "E", "Tem", "mu_fluid", "mu_e", "mu_sgs")
        hin = {k: getattr(dev, k).cpu().pin_memory() for k in ins}
        dins = [{k: getattr(dev, k) for k in ins}, {k: torch.empty_like(getattr(dev, k)) for k in ins}]
        douts = [[dev.Rmass, dev.Rmom, dev.Rener, dev.Dmass, dev.Dmom, dev.Dener],
                 [torch.empty_like(x) for x in (dev.Rmass, dev.Rmom, dev.Rener, dev.Dmass, dev.Dmom, dev.Dener)]]
        hout = [torch.empty(o.shape, dtype=o.dtype, pin_memory=True) for o in douts[0]]
        h2d = sum(v.numel() * v.element_size() for v in hin.values())
        d2h = sum(o.numel() * o.element_size() for o in douts[0])
        s_up, s_down = torch.cuda.Stream(device=device), torch.cuda.Stream(device=device)
        ev_in = [torch.cuda.Event() for _ in range(2)]
        ev_used = [torch.cuda.Event() for _ in range(2)]   # the kernels are done with input set b
        ev_done = [torch.cuda.Event() for _ in range(2)]   # the residuals of set b are on the host
        for e_ in ev_used + ev_done:
            e_.record(stream)
        geo = [cfg.porder, dev.nelem, dev.npoin, dev.connec.data_ptr(), None, None, dev.He.data_ptr(),
               dev.gpvol.data_ptr(), dev.dlxigp_ip.data_ptr(), None, dev.invAtoIJK.data_ptr(), dev.AtoI.data_ptr(),
               dev.AtoJ.data_ptr(), dev.AtoK.data_ptr()]

        def e2e_step(k):
            b = k % 2
            di, do = dins[b], douts[b]
            s_up.wait_event(ev_used[b])
            for name in ins:
                v = di[name]
                capi.check(L.msod_h2d(v.data_ptr(), hin[name].data_ptr(), v.numel() * v.element_size(),
                                      s_up.cuda_stream))
            ev_in[b].record(s_up)
            stream.wait_event(ev_in[b])
            stream.wait_event(ev_done[b])
            sc = stream.cuda_stream
            capi.check(L.msod_convec_ijk(*geo, di["u"].data_ptr(), di["q"].data_ptr(), di["rho"].data_ptr(),
                                         di["pr"].data_ptr(), di["E"].data_ptr(), do[0].data_ptr(),
                                         do[1].data_ptr(), do[2].data_ptr(), sc))
            capi.check(L.msod_diffusion_ijk(*geo, C.c_float(cfg.Cp), C.c_float(cfg.Pr), di["rho"].data_ptr(),
                                            di["u"].data_ptr(), di["Tem"].data_ptr(), di["mu_fluid"].data_ptr(),
                                            di["mu_e"].data_ptr(), di["mu_sgs"].data_ptr(), do[3].data_ptr(),
                                            do[4].data_ptr(), do[5].data_ptr(), sc))
            ev_used[b].record(stream)
            s_down.wait_event(ev_used[b])
            for o, h in zip(do, hout):
                capi.check(L.msod_d2h(h.data_ptr(), o.data_ptr(), o.numel() * o.element_size(), s_down.cuda_stream))
            ev_done[b].record(s_down)

        link = host_link([(dins[1][k].data_ptr(), hin[k].data_ptr(), hin[k].numel() * hin[k].element_size())
                          for k in ins],
                         [(o.data_ptr(), h.data_ptr(), o.numel() * o.element_size()) for o, h in zip(douts[1], hout)],
                         s_up, s_down)
        for k in range(args.warmup):
            e2e_step(k)
        torch.cuda.synchronize()
        barrier(world)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        s_up.wait_event(a)
        s_down.wait_event(a)
        for k in range(args.steps):
            e2e_step(k)
        stream.wait_stream(s_down)
        b.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        e2e_ms = max_over_ranks(a.elapsed_time(b), world, device) / args.steps
        e2e = {"value": world * 5.0 * dev.npoin / (e2e_ms * 1e-3) / 1e9, "unit": "GDOF/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
               "host_link": dict(link, floor_ms_per_step=link["both_ms"]),
               "path": "per step: msod_h2d x9 (pinned host -> device), msod_convec_ijk, msod_diffusion_ijk, "
                       "msod_d2h x6 (device -> pinned host); steps pipelined over two device buffer sets on three "
                       "streams (uploads of k+1 and downloads of k-1 overlap the kernels of k), fill and drain "
                       "inside the timed region"}
        del dins, douts

    if rank != 0:
        return
    peak, peak_kind = peak_hbm()
    dom = "convec" if conv_ms >= diff_ms else "diffu"
    dom_ms = conv_ms if dom == "convec" else diff_ms
    dom_b = Bc if dom == "convec" else Bd
    achieved = dom_b / (dom_ms * 1e-3) / 1e9
    tr = load_traffic(cfg.name) or {}
    traffic = tr.get("convec_ijk" if dom == "convec" else "diffusion_ijk")
    out = {
        "metric": METRIC, "value": value, "unit": "GDOF/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered structured mesh, Fourier fields)",
        "config": workload_config(cfg, dev.nelem, dev.npoin),
        "parallelism": "replica per GPU" if world > 1 else "single GPU",
        "roofline": {"bound": "hbm", "kernel": dom + " call (output zeroing + kernel)", "achieved": achieved,
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "algorithmic_bytes": dom_b},
        "kernels": {"convec_ms": conv_ms, "diffu_ms": diff_ms, "convec_gbs": Bc / conv_ms / 1e6,
                    "diffu_gbs": Bd / diff_ms / 1e6,
                    "combined_frac": (Bc + Bd) / ((conv_ms + diff_ms) * 1e-3) / 1e9 / peak},
        "gpu_launches": 4 * args.steps,  # per step: table preparation + kernel, for each of the two calls
        "clocks": clocks,
        "e2e": e2e,
    }
    if world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(cfg, host, args.cpu_seconds)
    if world == 1 and not args.no_variants:
        del dev
        out["variants"] = run_variants(host=host)
    print(json.dumps(out))


# --------------------------------------------------------------------------------------
# Variants beside the plain step: mixed precision and the learned viscosity
# --------------------------------------------------------------------------------------
def _ms(fn, reps):
    import torch

    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / reps


def _rel(a, b):
    import torch

    nb = float(torch.linalg.vector_norm(b.double()))
    d = float(torch.linalg.vector_norm((a.double() - b.double())))
    return d / nb if nb > 0 else d


def _fp64_runs(dev, mu_e=None):
    """The plain kernels' FP64 build (the GPU FP64 oracle run): the element tables in FP64, as the
    reference's FP64 build computes them (msod_fem_element_tables_f64), and the FP32 fields, He and
    gpvol promoted to FP64 -- the inputs every compared path shares.  (With the FP32 tables promoted
    instead, the reference run carries their rounding: the diffusion residual cancels so strongly
    that it moves by ~1e-3 relative on the 32^3 porder-7 workload.)"""
    import torch

    from minisod2d_gb300 import fem, kernels

    g = dev.geometry()
    d = lambda t: t.double()
    mk = lambda: (torch.empty(dev.npoin, dtype=torch.float64, device=dev.He.device),
                  torch.empty(3 * dev.npoin, dtype=torch.float64, device=dev.He.device),
                  torch.empty(dev.npoin, dtype=torch.float64, device=dev.He.device))
    dl64 = torch.from_numpy(fem.element_tables(dev.cfg.porder, np.float64)["dlxigp_ip"]).to(dev.He.device)
    geo = (g[0], g[1], g[2], None, None, d(dev.He), d(dev.gpvol), dl64, None, *g[9:])
    c64, d64 = mk(), mk()
    kernels.full_convec_ijk(*geo, d(dev.u), d(dev.q), d(dev.rho), d(dev.pr), d(dev.E), *c64)
    kernels.full_diffusion_ijk(*geo, dev.cfg.Cp, dev.cfg.Pr, d(dev.rho), d(dev.u), d(dev.Tem), d(dev.mu_fluid),
                               d(dev.mu_e if mu_e is None else mu_e), d(dev.mu_sgs), *d64)
    torch.cuda.synchronize()
    return c64, d64


def variant_mixed(reps):
    """mixed_p7: plain FP32 kernels against the FP16 / BF16 tensor-core kernels."""
    import torch

    from minisod2d_gb300 import workload

    cfg = workload.CONFIGS["mixed_p7"]
    dev = workload.DeviceCase(workload.HostCase(cfg))
    c64, d64 = _fp64_runs(dev)
    names = ("Rmass", "Rmom", "Rener")
    res = {"workload": "mixed_p7: 32^3 hexes, porder 7, +-5% jitter, 16-mode smooth fields",
           "error_reference": "FP64 build of the plain kernels on the same inputs"}
    pc, pd = _ms(lambda: dev.convec(), reps), _ms(lambda: dev.diffu(), reps)
    c32, d32 = dev.convec(), dev.diffu()
    res["plain_fp32"] = {"convec_ms": pc, "diffu_ms": pd,
                         "convec_err": {k: _rel(a, b) for k, a, b in zip(names, c32, c64)},
                         "diffu_err": {k: _rel(a, b) for k, a, b in zip(names, d32, d64)}}
    out = tuple(torch.empty_like(x) for x in c64)
    for prec in ("fp16", "bf16"):
        mc = _ms(lambda: dev.convec_mixed(prec, out=out), reps)
        ce = {k: _rel(a, b) for k, a, b in zip(names, dev.convec_mixed(prec, out=out), c64)}
        md = _ms(lambda: dev.diffu_mixed(prec, out=out), reps)
        de = {k: _rel(a, b) for k, a, b in zip(names, dev.diffu_mixed(prec, out=out), d64)}
        res[prec] = {"convec_ms": mc, "diffu_ms": md, "convec_err": ce, "diffu_err": de,
                     "speedup_vs_plain": (pc + pd) / (mc + md)}
    return res


def variant_learned(reps):
    """learned_48 on a held-out seed: the shipped network against the plain estimator."""
    from minisod2d_gb300 import learn, workload

    cfg = workload.CONFIGS["learned_48"]
    host = workload.HostCase(workload.Config(cfg.name, cfg.porder, cfg.nx, cfg.jitter, cfg.kind, cfg.nmodes, 2024))
    dev = workload.DeviceCase(host)
    m = learn.Mlp()
    m.load(learn.shipped_weights("learned_48"))
    r = learn.evaluate(m, dev, ybar=learn.shipped_report("learned_48")["ybar"], reps=reps)
    r["workload"] = "learned_48: 48^3 hexes, porder 4, shock-like fields, held-out seed 2024"
    r["speedup_estimator_plus_diffusion"] = r["ms_plain_estimator_plus_diffusion"] / \
        r["ms_learned_estimator_plus_diffusion"]
    return r


def variant_combined(reps):
    """combined_96: plain path (convection, entropy estimator, diffusion) against the
    learned path and the mixed + learned path."""
    import torch

    from minisod2d_gb300 import learn, workload

    cfg = workload.CONFIGS["combined_96"]
    dev = workload.DeviceCase(workload.HostCase(
        workload.Config(cfg.name, cfg.porder, cfg.nx, cfg.jitter, cfg.kind, cfg.nmodes, 2024)))  # held-out seed
    m = learn.Mlp()
    m.load(learn.shipped_weights("combined_96"))
    names = ("Rmass", "Rmom", "Rener")
    mu_p, nu_p, numax = learn.entropy_viscosity(dev)
    c64, d64 = _fp64_runs(dev, mu_e=mu_p)
    nu_l, flag = learn.learned_viscosity(m, dev)
    o64 = tuple(torch.empty_like(x) for x in c64)
    o64b = tuple(torch.empty_like(x) for x in c64)
    mu_buf = torch.empty_like(mu_p)

    def plain():
        dev.convec()
        learn.entropy_viscosity(dev, mu_buf, nu_p, numax)
        from minisod2d_gb300 import kernels
        kernels.full_diffusion_ijk(*dev.geometry(), cfg.Cp, cfg.Pr, dev.rho, dev.u, dev.Tem, dev.mu_fluid, mu_buf,
                                   dev.mu_sgs, dev.Dmass, dev.Dmom, dev.Dener)

    def learned32():
        dev.convec()
        learn.diffusion_learned(m, dev, nu=nu_l, flag=flag)

    def mixed_learned():
        dev.convec_mixed("fp16", out=o64)
        learn.learned_viscosity(m, dev, nu_l, flag)
        dev.diffu_mixed("fp16", nu_elem=nu_l, out=o64b)

    t_plain, t_l32, t_ml = _ms(plain, reps), _ms(learned32, reps), _ms(mixed_learned, reps)
    plain()
    pe = {"convec": {k: _rel(a, b) for k, a, b in zip(names, (dev.Rmass, dev.Rmom, dev.Rener), c64)},
          "diffu": {k: _rel(a, b) for k, a, b in zip(names, (dev.Dmass, dev.Dmom, dev.Dener), d64)}}
    learned32()
    le = {"diffu": {k: _rel(a, b) for k, a, b in zip(names, (dev.Dmass, dev.Dmom, dev.Dener), d64)}}
    mixed_learned()
    me = {"convec": {k: _rel(a, b) for k, a, b in zip(names, o64, c64)},
          "diffu": {k: _rel(a, b) for k, a, b in zip(names, o64b, d64)}}
    dofs = 5.0 * dev.npoin
    return {"workload": "combined_96: 96^3 hexes, porder 5, +-5% jitter, shock-like fields, held-out seed 2024; "
                        "network trained on 16 other seeds of this workload",
            "error_reference": "FP64 build of the plain kernels on the same inputs, diffusion with the plain "
                               "estimator's mu_e",
            "plain": {"ms": t_plain, "gdofs": dofs / t_plain / 1e6, "err": pe},
            "learned_fp32": {"ms": t_l32, "gdofs": dofs / t_l32 / 1e6, "err": le, "speedup": t_plain / t_l32,
                             "path": "convection + msod_diffusion_ijk_learned (features kernel with the network, "
                                     "fallback estimator on the flagged elements, per-element-viscosity diffusion)"},
            "mixed_fp16_learned": {"ms": t_ml, "gdofs": dofs / t_ml / 1e6, "err": me, "speedup": t_plain / t_ml},
            "fallback_fraction": float(flag.float().mean()),
            "nu_rel_l2_learned_vs_plain": _rel(nu_l, nu_p)}


def variant_tet(reps, host):
    """tet_64: the driver's TET04 kernels (fem_convec, fem_diffu) on its
    disconnected unit tetrahedra over the plain_64 node fields; errors against
    the FP64 build of the same kernels on the same inputs."""
    import torch

    from minisod2d_gb300 import workload

    tc = workload.TetCase(host)
    peak, kind = peak_hbm()
    res = {"workload": "tet_64: %d disconnected unit tetrahedra (the reference driver's TET04 mesh, "
                       "mod_mesh.f90:71-126), %d nodes carrying the plain_64 fields, mu_e = mu_sgs = 1, "
                       "Cp = Pr = 1" % (tc.nelem, tc.npoin),
           "assembly": "red.global.add.v4.f32 (nodes 4k..4k+3)",
           "error_reference": "FP64 build of the tet kernels on the same inputs"}
    names = ("Rmass", "Rmom", "Rener")
    t64 = workload.TetCase(host, dtype=torch.float64)
    for which in ("convec", "diffu"):
        fn32, fn64 = getattr(tc, which), getattr(t64, which)
        ms = _ms(fn32, reps)
        gbs = tc.algorithmic_bytes(which) / (ms * 1e-3) / 1e9
        a, b = fn32(), fn64()
        res[which] = {"ms": ms, "gbs": gbs, "frac": gbs / peak, "peak_gbs": peak, "peak_kind": kind,
                      "algorithmic_bytes": tc.algorithmic_bytes(which),
                      "err": {k: _rel(x, y) for k, x, y in zip(names, a, b)}}
    del t64
    return res


def variant_rk4(reps, host):
    """rk4_64: one explicit RK4 step (four stages of convection + diffusion through the C ABI, the
    lumped mass, the stage updates) on the plain_64 state, against four plain steps."""
    from minisod2d_gb300 import timestep, workload

    dev = workload.DeviceCase(host)
    Ml = timestep.lumped_mass(dev)
    ws = timestep.workspace(dev)
    rho, q, rhoE = dev.rho.clone(), dev.q.clone(), (dev.rho * dev.E).contiguous()
    t = _ms(lambda: timestep.rk4_step(dev, Ml, 1e-4, rho, q, rhoE, ws), reps)
    tp = _ms(lambda: (dev.convec(), dev.diffu()), reps)
    return {"workload": "rk4_64: the plain_64 state (rho, q = rho u, rhoE), dt = 1e-4, mu_e = mu_sgs = 0",
            "ms_per_step": t, "gdofs": 5.0 * dev.npoin / (t * 1e-3) / 1e9, "four_plain_steps_ms": 4.0 * tp,
            "stage_overhead_ms": t - 4.0 * tp, "workspace_bytes": int(ws.numel())}


def porder_sweep(reps=20, porders=range(1, 9), nodes_1d=256):
    """Both plain kernels at each porder on a structured mesh of nx = nodes_1d / porder hexes a side
    (about 16.8 M nodes at every porder, +-5 % jitter, smooth fields): time per call, GDOF/s and the
    fraction of the HBM copy peak of the compulsory bytes (every input read once, every output
    written once), and the time of the one-call form (msod_convec_diffusion_ijk).  Every working
    set is far above L2."""
    import torch

    from minisod2d_gb300 import workload

    peak, kind = peak_hbm()
    rows = []
    for P in porders:
        nx = int(round(nodes_1d / P))
        dev = workload.DeviceCase(workload.HostCase(workload.custom(P, nx, 0.05)))
        cb, db = algorithmic_bytes(dev.nelem, dev.cfg.nnode, dev.npoin)
        tc, td = _ms(lambda: dev.convec(), reps), _ms(lambda: dev.diffu(), reps)
        tf = _ms(lambda: dev.convec_diffu(), reps)
        dofs = 5.0 * dev.npoin
        rows.append({"porder": P, "nx": nx, "nelem": dev.nelem, "npoin": dev.npoin,
                     "convec_ms": tc, "diffu_ms": td, "gdofs": dofs / ((tc + td) * 1e-3) / 1e9,
                     "one_call_ms": tf, "one_call_gdofs": dofs / (tf * 1e-3) / 1e9,
                     "convec_frac": cb / (tc * 1e-3) / 1e9 / peak, "diffu_frac": db / (td * 1e-3) / 1e9 / peak,
                     "bytes_per_node": (cb + db) / dev.npoin})
        del dev
        torch.cuda.empty_cache()
    return {"porder_sweep": rows, "peak_gbs": peak, "peak_kind": kind,
            "workload": "structured hex meshes, nx = round(%d / porder) a side, +-5%% jitter, smooth fields "
                        "(8 modes), seed 0; FP32; inputs above L2" % nodes_1d}


def variant_fused(reps, host):
    """fused_64: the plain_64 step as the two drop-in calls and as one msod_convec_diffusion_ijk
    call (one kernel at porder 4), with the agreement of the two forms' residuals."""
    from minisod2d_gb300 import workload

    dev = workload.DeviceCase(host)
    ts = _ms(lambda: (dev.convec(), dev.diffu()), reps)
    sep = [x.clone() for x in dev.convec()] + [x.clone() for x in dev.diffu()]
    tf = _ms(lambda: dev.convec_diffu(), reps)
    c, d = dev.convec_diffu()
    names = ("convec_Rmass", "convec_Rmom", "convec_Rener", "diffu_Rmass", "diffu_Rmom", "diffu_Rener")
    dofs = 5.0 * dev.npoin
    return {"workload": "fused_64: the plain_64 inputs", "two_calls_ms": ts, "one_call_ms": tf,
            "two_calls_gdofs": dofs / (ts * 1e-3) / 1e9, "one_call_gdofs": dofs / (tf * 1e-3) / 1e9,
            "speedup": ts / tf, "rel_l2_one_vs_two": {k: _rel(a, b) for k, a, b in zip(names, c + d, sep)}}


def run_variants(reps=10, host=None):
    out = {}
    variants = [("mixed_p7", variant_mixed), ("learned_48", variant_learned), ("combined_96", variant_combined)]
    if host is not None:
        variants.insert(0, ("tet_64", lambda r: variant_tet(r, host)))
        variants.insert(1, ("rk4_64", lambda r: variant_rk4(r, host)))
        variants.insert(2, ("fused_64", lambda r: variant_fused(r, host)))
    for name, fn in variants:
        import torch

        try:
            out[name] = fn(reps)
        except Exception as ex:  # a variant never costs the plain measurement
            out[name] = {"error": "%s: %s" % (type(ex).__name__, ex)}
        torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="plain_64")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the mixed-precision / learned-viscosity measurements beside the plain step")
    ap.add_argument("--porder-sweep", action="store_true",
                    help="only time both plain kernels at porders 1-8 on meshes of about 16.8 M nodes")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)  # the timing rules ask for at least 3 warm-up steps
    from minisod2d_gb300 import workload

    if args.porder_sweep:
        print(json.dumps(porder_sweep()))
        return

    cfg = workload.CONFIGS[args.config]
    rank, local, world = dist_setup()
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, cfg)
        return
    run_ours(args, cfg, rank, local, world)


if __name__ == "__main__":
    main()
