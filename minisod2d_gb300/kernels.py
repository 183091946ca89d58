"""Python mirror of the reference's hot-path subroutines over CUDA tensors.

``full_convec_ijk``, ``full_convec_ijk_split`` and ``full_diffusion_ijk`` take
the reference's arguments in the reference's order (elem_convec.f90:198,
:433; elem_diffu.f90:10) as CUDA tensors in the reference's column-major
layouts flattened to 1-D, write the intent(out) residuals in place and run
on torch's current stream through the C ABI (libmsod.so).  There is no CPU
path: a tensor on another device is an error.
"""
from . import capi


def _stream(stream):
    if stream is not None:
        return stream
    import torch

    return torch.cuda.current_stream().cuda_stream


def _porder_from(gmshAtoI):
    n = int(gmshAtoI.numel())
    q = int(round(n ** (1.0 / 3.0)))
    if q ** 3 != n or q < 2:
        raise ValueError("gmshAtoI has %d entries, not (porder+1)^3" % n)
    return q - 1


def _ptr(t, name, dtype, numel=None):
    import torch

    if t is None:
        return None
    if not isinstance(t, torch.Tensor):
        raise TypeError("%s must be a torch tensor" % name)
    if not t.is_cuda:
        raise ValueError("%s must be a CUDA tensor (the library has no CPU path)" % name)
    if t.dtype != dtype:
        raise TypeError("%s must be %s, got %s" % (name, dtype, t.dtype))
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    if numel is not None and t.numel() != numel:
        raise ValueError("%s has %d elements, expected %d" % (name, t.numel(), numel))
    return t.data_ptr()


def _geometry(nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, real):
    import torch

    P = _porder_from(gmshAtoI)
    n = (P + 1) ** 3
    return P, [
        _ptr(connec, "connec", torch.int32, nelem * n),
        _ptr(He, "He", real, 9 * nelem * n),
        _ptr(gpvol, "gpvol", real, nelem * n),
        _ptr(dlxigp_ip, "dlxigp_ip", real, 3 * n * (P + 1)),
        _ptr(invAtoIJK, "invAtoIJK", torch.int32, n),
        _ptr(gmshAtoI, "gmshAtoI", torch.int32, n),
        _ptr(gmshAtoJ, "gmshAtoJ", torch.int32, n),
        _ptr(gmshAtoK, "gmshAtoK", torch.int32, n),
    ]


def full_convec_ijk(nelem, npoin, connec, Ngp, dNgp, He, gpvol, dlxigp_ip, xgp, invAtoIJK, gmshAtoI, gmshAtoJ,
                    gmshAtoK, u, q, rho, pr, E, Rmass, Rmom, Rener, stream=None, split=False):
    """elem_convec.f90:198 (``split=True``: :433).  Ngp, dNgp, xgp are ignored."""
    import torch

    real = He.dtype
    P, g = _geometry(nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, real)
    f = [_ptr(u, "u", real, 3 * npoin), _ptr(q, "q", real, 3 * npoin), _ptr(rho, "rho", real, npoin),
         _ptr(pr, "pr", real, npoin), _ptr(E, "E", real, npoin), _ptr(Rmass, "Rmass", real, npoin),
         _ptr(Rmom, "Rmom", real, 3 * npoin), _ptr(Rener, "Rener", real, npoin)]
    st = _stream(stream)
    if real == torch.float32:
        name = "msod_convec_ijk_split" if split else "msod_convec_ijk"
        capi.call(name, P, nelem, npoin, g[0], None, None, g[1], g[2], g[3], None, *g[4:], *f, st)
    elif real == torch.float64:
        capi.call("msod_convec_ijk_f64", P, nelem, npoin, *g, *f, st)
    else:
        raise TypeError("He must be float32 or float64")


def full_convec_ijk_split(*args, **kw):
    """elem_convec.f90:433 -- same arguments and residuals as full_convec_ijk."""
    kw["split"] = True
    return full_convec_ijk(*args, **kw)


def full_diffusion_ijk(nelem, npoin, connec, Ngp, dNgp, He, gpvol, dlxigp_ip, xgp, invAtoIJK, gmshAtoI, gmshAtoJ,
                       gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener, stream=None):
    """elem_diffu.f90:10.  Ngp, dNgp, xgp are ignored."""
    import torch

    real = He.dtype
    P, g = _geometry(nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, real)
    n = (P + 1) ** 3
    f = [_ptr(rho, "rho", real, npoin), _ptr(u, "u", real, 3 * npoin), _ptr(Tem, "Tem", real, npoin),
         _ptr(mu_fluid, "mu_fluid", real, npoin), _ptr(mu_e, "mu_e", real, nelem * n),
         _ptr(mu_sgs, "mu_sgs", real, nelem * n), _ptr(Rmass, "Rmass", real, npoin),
         _ptr(Rmom, "Rmom", real, 3 * npoin), _ptr(Rener, "Rener", real, npoin)]
    st = _stream(stream)
    if real == torch.float32:
        capi.call("msod_diffusion_ijk", P, nelem, npoin, g[0], None, None, g[1], g[2], g[3], None, *g[4:],
                  float(Cp), float(Pr), *f, st)
    elif real == torch.float64:
        capi.call("msod_diffusion_ijk_f64", P, nelem, npoin, *g, float(Cp), float(Pr), *f, st)
    else:
        raise TypeError("He must be float32 or float64")


def full_convec_diffusion_ijk(nelem, npoin, connec, Ngp, dNgp, He, gpvol, dlxigp_ip, xgp, invAtoIJK, gmshAtoI,
                              gmshAtoJ, gmshAtoK, Cp, Pr, u, q, rho, pr, E, Tem, mu_fluid, mu_e, mu_sgs, Rmass_c,
                              Rmom_c, Rener_c, Rmass_d, Rmom_d, Rener_d, stream=None):
    """full_convec_ijk (elem_convec.f90:198) and full_diffusion_ijk (elem_diffu.f90:10) of the same
    geometry and state in one call (msod_convec_diffusion_ijk, FP32).  Ngp, dNgp, xgp are ignored."""
    import torch

    real = He.dtype
    if real != torch.float32:
        raise TypeError("He must be float32")
    P, g = _geometry(nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, real)
    n = (P + 1) ** 3
    f = [_ptr(u, "u", real, 3 * npoin), _ptr(q, "q", real, 3 * npoin), _ptr(rho, "rho", real, npoin),
         _ptr(pr, "pr", real, npoin), _ptr(E, "E", real, npoin), _ptr(Tem, "Tem", real, npoin),
         _ptr(mu_fluid, "mu_fluid", real, npoin), _ptr(mu_e, "mu_e", real, nelem * n),
         _ptr(mu_sgs, "mu_sgs", real, nelem * n)]
    r = [_ptr(Rmass_c, "Rmass_c", real, npoin), _ptr(Rmom_c, "Rmom_c", real, 3 * npoin),
         _ptr(Rener_c, "Rener_c", real, npoin), _ptr(Rmass_d, "Rmass_d", real, npoin),
         _ptr(Rmom_d, "Rmom_d", real, 3 * npoin), _ptr(Rener_d, "Rener_d", real, npoin)]
    capi.call("msod_convec_diffusion_ijk", P, nelem, npoin, g[0], None, None, g[1], g[2], g[3], None, *g[4:],
              float(Cp), float(Pr), *f, *r, _stream(stream))


def full_convec_ijk_mixed(nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                          u, q, rho, pr, E, Rmass, Rmom, Rener, precision="fp16", stream=None):
    """Mixed-precision form of elem_convec.f90:198: FP32 fields, FP64 residuals.

    ``precision`` is "fp16" or "bf16" (hi + lo split tensor-core contractions).
    """
    import torch

    P, g = _geometry(nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                     torch.float32)
    f = [_ptr(u, "u", torch.float32, 3 * npoin), _ptr(q, "q", torch.float32, 3 * npoin),
         _ptr(rho, "rho", torch.float32, npoin), _ptr(pr, "pr", torch.float32, npoin),
         _ptr(E, "E", torch.float32, npoin), _ptr(Rmass, "Rmass", torch.float64, npoin),
         _ptr(Rmom, "Rmom", torch.float64, 3 * npoin), _ptr(Rener, "Rener", torch.float64, npoin)]
    prec = {"fp16": capi.MSOD_PREC_FP16, "bf16": capi.MSOD_PREC_BF16}[precision]
    capi.call("msod_convec_ijk_mixed", prec, P, nelem, npoin, *g, *f, _stream(stream))


def full_diffusion_ijk_mixed(nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                             Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener, precision="fp16",
                             nu_elem=None, stream=None):
    """Mixed-precision form of elem_diffu.f90:10: FP32 fields, FP64 residuals.

    With ``nu_elem`` (one value per element) mu_e(e, a) = rho(a) nu_elem(e)
    and ``mu_e`` is ignored."""
    import torch

    P, g = _geometry(nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                     torch.float32)
    n = (P + 1) ** 3
    visc = _ptr(nu_elem, "nu_elem", torch.float32, nelem) if nu_elem is not None else \
        _ptr(mu_e, "mu_e", torch.float32, nelem * n)
    f = [_ptr(rho, "rho", torch.float32, npoin), _ptr(u, "u", torch.float32, 3 * npoin),
         _ptr(Tem, "Tem", torch.float32, npoin), _ptr(mu_fluid, "mu_fluid", torch.float32, npoin), visc,
         _ptr(mu_sgs, "mu_sgs", torch.float32, nelem * n), _ptr(Rmass, "Rmass", torch.float64, npoin),
         _ptr(Rmom, "Rmom", torch.float64, 3 * npoin), _ptr(Rener, "Rener", torch.float64, npoin)]
    prec = {"fp16": capi.MSOD_PREC_FP16, "bf16": capi.MSOD_PREC_BF16}[precision]
    name = "msod_diffusion_ijk_mixed_nu" if nu_elem is not None else "msod_diffusion_ijk_mixed"
    capi.call(name, prec, P, nelem, npoin, *g, float(Cp), float(Pr), *f, _stream(stream))


def elem_jacobian(porder, nelem, npoin, connec, coord, dNgp, wgp, gpvol, He, stream=None):
    """jacobian_oper.f90:7 on the device; writes gpvol and He in place."""
    import torch

    real = coord.dtype
    n = (porder + 1) ** 3
    args = [_ptr(connec, "connec", torch.int32, nelem * n), _ptr(coord, "coord", real, 3 * npoin),
            _ptr(dNgp, "dNgp", real, 3 * n * n), _ptr(wgp, "wgp", real, n), _ptr(gpvol, "gpvol", real, nelem * n),
            _ptr(He, "He", real, 9 * nelem * n)]
    name = "msod_elem_jacobian" if real == torch.float32 else "msod_elem_jacobian_f64"
    capi.call(name, int(porder), nelem, npoin, *args, _stream(stream))


def _tet_geometry(nelem, connec, Ngp, dNgp, He, gpvol, real):
    import torch

    return [_ptr(connec, "connec", torch.int32, 4 * nelem), _ptr(Ngp, "Ngp", real, 16),
            _ptr(dNgp, "dNgp", real, 48), _ptr(He, "He", real, 36 * nelem), _ptr(gpvol, "gpvol", real, 4 * nelem)]


def fem_convec(nelem, npoin, connec, Ngp, dNgp, He, gpvol, u, q, rho, pr, E, Rmass, Rmom, Rener, stream=None):
    """elem_convec.f90:839 (linear tetrahedra)."""
    import torch

    real = He.dtype
    g = _tet_geometry(nelem, connec, Ngp, dNgp, He, gpvol, real)
    f = [_ptr(u, "u", real, 3 * npoin), _ptr(q, "q", real, 3 * npoin), _ptr(rho, "rho", real, npoin),
         _ptr(pr, "pr", real, npoin), _ptr(E, "E", real, npoin), _ptr(Rmass, "Rmass", real, npoin),
         _ptr(Rmom, "Rmom", real, 3 * npoin), _ptr(Rener, "Rener", real, npoin)]
    if real not in (torch.float32, torch.float64):
        raise TypeError("He must be float32 or float64")
    name = "msod_fem_convec" if real == torch.float32 else "msod_fem_convec_f64"
    capi.call(name, nelem, npoin, *g, *f, _stream(stream))


def fem_diffu(nelem, npoin, connec, Ngp, dNgp, He, gpvol, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs, Rmass, Rmom,
              Rener, stream=None):
    """elem_diffu.f90:199 (linear tetrahedra)."""
    import torch

    real = He.dtype
    g = _tet_geometry(nelem, connec, Ngp, dNgp, He, gpvol, real)
    f = [_ptr(rho, "rho", real, npoin), _ptr(u, "u", real, 3 * npoin), _ptr(Tem, "Tem", real, npoin),
         _ptr(mu_fluid, "mu_fluid", real, npoin), _ptr(mu_e, "mu_e", real, 4 * nelem),
         _ptr(mu_sgs, "mu_sgs", real, 4 * nelem), _ptr(Rmass, "Rmass", real, npoin),
         _ptr(Rmom, "Rmom", real, 3 * npoin), _ptr(Rener, "Rener", real, npoin)]
    if real not in (torch.float32, torch.float64):
        raise TypeError("He must be float32 or float64")
    name = "msod_fem_diffu" if real == torch.float32 else "msod_fem_diffu_f64"
    capi.call(name, nelem, npoin, *g, float(Cp), float(Pr), *f, _stream(stream))


def tet_jacobian(nelem, npoin, connec, coord, dNgp, wgp, gpvol, He, stream=None):
    """jacobian_oper.f90:138 on the device; writes gpvol and He in place."""
    import torch

    real = coord.dtype
    args = [_ptr(connec, "connec", torch.int32, 4 * nelem), _ptr(coord, "coord", real, 3 * npoin),
            _ptr(dNgp, "dNgp", real, 48), _ptr(wgp, "wgp", real, 4), _ptr(gpvol, "gpvol", real, 4 * nelem),
            _ptr(He, "He", real, 36 * nelem)]
    name = "msod_tet_jacobian" if real == torch.float32 else "msod_tet_jacobian_f64"
    capi.call(name, nelem, npoin, *args, _stream(stream))


def check_element_tables(porder, nelem, npoin, connec, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                         stream=None):
    import torch

    n = (porder + 1) ** 3
    capi.call("msod_check_element_tables", int(porder), nelem, npoin,
              _ptr(connec, "connec", torch.int32, nelem * n), _ptr(dlxigp_ip, "dlxigp_ip", torch.float32),
              _ptr(invAtoIJK, "invAtoIJK", torch.int32, n), _ptr(gmshAtoI, "gmshAtoI", torch.int32, n),
              _ptr(gmshAtoJ, "gmshAtoJ", torch.int32, n), _ptr(gmshAtoK, "gmshAtoK", torch.int32, n),
              _stream(stream))


def set_checked(enabled):
    capi.call("msod_set_checked", 1 if enabled else 0)


def set_mode(precision="fp32", mu_e="given", mlp=None):
    """The form of every later full_convec_ijk / full_diffusion_ijk call
    (msod_set_mode): precision "fp32", "fp16" or "bf16"; mu_e "given",
    "plain" (entropy-viscosity estimator) or "learned" (``mlp``, a learn.Mlp)."""
    prec = {"fp32": capi.MSOD_PREC_FP32, "fp16": capi.MSOD_PREC_FP16, "bf16": capi.MSOD_PREC_BF16}[precision]
    mue = {"given": capi.MSOD_MU_E_GIVEN, "plain": capi.MSOD_MU_E_PLAIN, "learned": capi.MSOD_MU_E_LEARNED}[mu_e]
    capi.call("msod_set_mode", prec, mue, mlp.h if mlp is not None else None)


def get_mode():
    import ctypes as C

    p, m = C.c_int(), C.c_int()
    capi.call("msod_get_mode", C.byref(p), C.byref(m))
    return ({capi.MSOD_PREC_FP32: "fp32", capi.MSOD_PREC_FP16: "fp16", capi.MSOD_PREC_BF16: "bf16"}[p.value],
            {capi.MSOD_MU_E_GIVEN: "given", capi.MSOD_MU_E_PLAIN: "plain", capi.MSOD_MU_E_LEARNED: "learned"}[m.value])


__all__ = ["full_convec_ijk", "full_convec_ijk_split", "full_diffusion_ijk", "full_convec_ijk_mixed",
           "full_diffusion_ijk_mixed", "elem_jacobian", "set_mode", "get_mode",
           "check_element_tables", "set_checked"]
