"""The reference's exported kernel functions (src/GPUCellListSPH.jl:15-17) over
libgcsph.so.  Arguments follow the Julia signatures (src/gpukernels_sph.jl);
vector arguments are tuples of D CUDA float64 tensors, `pairs` is an (P, 2)
int32 CUDA tensor of 1-based pairs.  Python names: sph∇W! -> sphgradW,
sph∑W! -> sphsumW, sph∑∇W! -> sphsumgradW, ∂ρ∂tDDT! -> drhodtDDT,
∂v∂t! -> dvdt, ∂v∂t_av! -> dvdt_av, ∂v∂t_visc! -> dvdt_visc,
∂v∂t_addgrav! -> dvdt_addgrav, ∂v∂tpF! -> dvdtpF.
"""
from __future__ import annotations

import ctypes as C

from . import _lib


def _D(vec):
    return len(vec)


def _N(vec):
    return int(vec[0].numel())


def _P(pairs):
    return int(pairs.shape[0]) if pairs is not None else 0


def _p(t):
    return _lib.dptr(t)


def _v(vec):
    return _lib.ptrs(vec)


def sphW(W, pairs, points, Hinv, sphkernel=None):
    """sphW!(W, pairs, points, H⁻¹, sphkernel) -- :75-100"""
    _lib.check(_lib.load().gcsph_sphW(_D(points), _N(points), _P(pairs), _p(pairs), _v(points), float(Hinv), _p(W),
                                      None))


def sphgradW(gW, pairs, points, Hinv, sphkernel=None):
    """sph∇W!(∇W, pairs, points, H⁻¹, kernel) -- :186-213"""
    _lib.check(_lib.load().gcsph_sphgradW(_D(points), _N(points), _P(pairs), _p(pairs), _v(points), float(Hinv),
                                          _v(gW), None))


def sphsumW(sumW, pairs, points, sphkernel, Hinv, ptype):
    """sph∑W!(∑W, pairs, points, sphkernel, H⁻¹, ptype) -- :129-156"""
    _lib.check(_lib.load().gcsph_sphsumW(_D(points), _N(points), _P(pairs), _p(pairs), _v(points), float(Hinv),
                                         _p(ptype), _p(sumW), None))


def sphsumgradW(sumgW, pairs, points, sphkernel, Hinv, ptype):
    """sph∑∇W!(∑∇W, pairs, points, kernel, H⁻¹, ptype) -- :322-359"""
    _lib.check(_lib.load().gcsph_sphsumgradW(_D(points), _N(points), _P(pairs), _p(pairs), _v(points), float(Hinv),
                                             _p(ptype), _v(sumgW), None))


def drhodtDDT(drhodt, pairs, gW, rho, v, points, h, m0, rho0, c0, gamma, g, delta, ptype):
    """∂ρ∂tDDT!(∑∂ρ∂t, pairs, ∇W, ρ, v, points, h, m₀, ρ₀, c₀, γ, g, δᵩ, ptype) -- :542-631"""
    _lib.check(_lib.load().gcsph_drhodt_ddt(_D(points), _N(points), _P(pairs), _p(pairs), _v(gW), _p(rho), _v(v),
                                            _v(points), float(h), float(m0), float(rho0), float(c0), int(gamma),
                                            float(g), float(delta), _p(ptype), _p(drhodt), None))


def pressure(P, rho, c0, gamma, rho0, ptype):
    """pressure!(P, ρ, c₀, γ, ρ₀, ptype) -- :710-727"""
    if not (P.numel() == rho.numel() == ptype.numel()):
        raise ValueError("Wrong length")
    _lib.check(_lib.load().gcsph_pressure(int(rho.numel()), _p(rho), float(c0), int(gamma), float(rho0), _p(ptype),
                                          _p(P), None))


def dvdt(a, gW, P, pairs, m0, rho, ptype):
    """∂v∂t!(∑∂v∂t, ∇W, P, pairs, m₀, ρ, ptype) -- :740-776"""
    _lib.check(_lib.load().gcsph_dvdt(_D(a), _N(a), _P(pairs), _p(pairs), _v(gW), _p(P), float(m0), _p(rho),
                                      _p(ptype), _v(a), None))


def dvdt_av(a, gW, pairs, points, h, rho, alpha, v, c0, m0, ptype):
    """∂v∂t_av!(∑∂v∂t, ∇W, pairs, points, h, ρ, α, v, c₀, m₀, ptype) -- :852-901"""
    _lib.check(_lib.load().gcsph_dvdt_av(_D(a), _N(a), _P(pairs), _p(pairs), _v(gW), _v(points), float(h), _p(rho),
                                         float(alpha), _v(v), float(c0), float(m0), _p(ptype), _v(a), None))


def dvdt_visc(a, gW, v, rho, points, pairs, h, m0, nu, ptype):
    """∂v∂t_visc!(∑∂v∂t, ∇W, v, ρ, points, pairs, h, m₀, 𝜈, ptype) -- :952-991"""
    _lib.check(_lib.load().gcsph_dvdt_visc(_D(a), _N(a), _P(pairs), _p(pairs), _v(gW), _v(v), _p(rho), _v(points),
                                           float(h), float(m0), float(nu), _p(ptype), _v(a), None))


def dvdt_addgrav(a, g):
    """∂v∂t_addgrav!(∑∂v∂t, gravvec(g, dim)) -- :1031-1051"""
    _lib.check(_lib.load().gcsph_addgrav(_D(a), _N(a), float(g), _v(a), None))


def fbmolforce(a, pairs, points, d, r0, ptype):
    """fbmolforce!(∑∂v∂t, pairs, points, d, r₀, ptype) -- :1875-1913"""
    _lib.check(_lib.load().gcsph_fbmolforce(_D(a), _N(a), _P(pairs), _p(pairs), _v(points), float(d), float(r0),
                                            _p(ptype), _v(a), None))


def dvdtpF(a, pairs, points, s, h, m0, ptype):
    """∂v∂tpF!(∑∂v∂t, pairs, points, s, h, m₀, ptype) -- :1373-1409"""
    _lib.check(_lib.load().gcsph_dvdt_pF(_D(a), _N(a), _P(pairs), _p(pairs), _v(points), float(s), float(h),
                                         float(m0), _p(ptype), _v(a), None))


def update_rho(rho, drhodt, dt, rho0, ptype):
    """update_ρp∂ρ∂tΔt!(ρ, ∑∂ρ∂t, Δt, ρ₀, ptype) -- :1078-1096"""
    if rho.numel() != drhodt.numel():
        raise ValueError("Wrong length")
    _lib.check(_lib.load().gcsph_update_rho(int(rho.numel()), _p(rho), _p(drhodt), float(dt), float(rho0),
                                            _p(ptype), None))


def update_v(v, a, dt, ptype):
    """update_vp∂v∂tΔt!(v, ∑∂v∂t, Δt, ptype) -- :1107-1127"""
    _lib.check(_lib.load().gcsph_update_v(_D(v), _N(v), _v(v), _v(a), float(dt), _p(ptype), None))


def update_x(x, v, dt):
    """update_xpvΔt!(x, v, Δt) -- :1150-1169"""
    _lib.check(_lib.load().gcsph_update_x(_D(x), _N(x), _v(x), _v(v), float(dt), None))


def symplectic_update(rho, rhoh, v, vh, x, xh, drhodt, a, dt, cdx, rho0, ptype):
    """symplectic_update!(ρ, ρΔt½, v, vΔt½, x, xΔt½, ∑∂ρ∂t, ∑∂v∂t, Δt, cΔx, ρ₀, ptype) -- :1193-1245"""
    _lib.check(_lib.load().gcsph_symplectic(_D(x), _N(x), _p(rho), _p(rhoh), _v(v), _v(vh), _v(x), _v(xh),
                                            _p(drhodt), _v(a), float(dt), _v(cdx), float(rho0), _p(ptype), None))


def dpcreg(buf, v, rho, P, pairs, points, sphkernel, l0, Pmin, Pmax, dt, lam, dpckernlim, ptype):
    """dpcreg!(∑Δvdpc, v, ρ, P, pairs, points, kernel, l₀, Pmin, Pmax, Δt, λ, dpckernlim, ptype) -- :1485-1553"""
    _lib.check(_lib.load().gcsph_dpcreg(_D(points), _N(points), _P(pairs), _v(buf), _v(v), _p(rho), _p(P),
                                        _p(pairs), _v(points), float(l0), float(Pmin), float(Pmax), float(dt),
                                        float(lam), float(dpckernlim), _p(ptype), None))


def update_dpcreg(v, x, buf, dt, ptype):
    """update_dpcreg!(v, x, ∑Δvdpc, Δt, ptype) -- :1607-1632"""
    _lib.check(_lib.load().gcsph_update_dpcreg(_D(x), _N(x), _v(v), _v(x), _v(buf), float(dt), _p(ptype), None))


def xsphcorr(buf, pairs, W, rho, v, m0, eps, ptype):
    """xsphcorr!(∑Δvxsph, pairs, W, ρ, v, m₀, 𝜀, ptype) -- :1745-1779"""
    _lib.check(_lib.load().gcsph_xsphcorr(_D(v), _N(v), _P(pairs), _v(buf), _p(pairs), _p(W), _p(rho), _v(v),
                                          float(m0), float(eps), _p(ptype), None))


def update_xsphcorr(x, buf, dt, ptype):
    """update_xsphcorr!(x, ∑Δvxsph, Δt, ptype) -- :1817-1838"""
    _lib.check(_lib.load().gcsph_update_xsph(_D(x), _N(x), _v(x), _v(buf), float(dt), _p(ptype), None))


def cspmcorr(buf, W, rho, m0, pairs, ptype):
    """cspmcorr!(∑ρcspm, W, ρ, m₀, pairs, ptype) -- :1673-1719"""
    _lib.check(_lib.load().gcsph_cspmcorr(_D(buf), int(rho.numel()), _P(pairs), _v(buf), _p(W), _p(rho), float(m0),
                                          _p(pairs), _p(ptype), None))


def dt_stepping(a, v, points, c0, h, CFL, timelims):
    """Δt_stepping(buf, a, v, points, c₀, h, CFL, timelims) -- :1293-1353; returns Δt"""
    out = C.c_double()
    _lib.check(_lib.load().gcsph_dt_stepping(_D(points), _N(points), _v(a), _v(v), _v(points), float(c0), float(h),
                                             float(CFL), float(timelims[0]), float(timelims[1]), C.byref(out), None))
    return float(out.value)


def dpckernlim(dim: int) -> float:
    """find_zero(x -> 1 - 𝒲(WendlandC2, x, 1), 0.5) -- src/sphproblem.jl:218"""
    return float(_lib.load().gcsph_dpckernlim(int(dim)))
