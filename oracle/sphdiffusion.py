"""Analytic diffusion solution for a sphere inside an infinite slab -- test
infrastructure (an independent physics check of the photon engine), not part
of the product.

Restates the reference's sphere-diffusion toolbox (matlab/sphdiffusionslab.m,
sphdiffusionsemi.m, sphdiffusioninfinite.m, sphdiffusionscatteronly.m,
sphdiffincident.m, sphdiffscatter.m, sphdiffinterior.m, sphdiffAcoeff.m,
sphdiffBcoeff.m, sphdiffCcoeff.m) for a source on the sphere's axis (polar
angle 0 or pi), where only the m = 0 harmonics contribute (sphdiffAcoeff.m
and sphdiffCcoeff.m return 0 for m != 0 there), so the field is a Legendre
series in cos(theta).

Physics (continuous wave when omega = 0): a point source at distance R_s from
the centre of a sphere of radius a; outside, the fluence is the incident
Green's function v/(4 pi D_out d) exp(i k_out d) plus the scattered series
sum_l (A_l j_l(k_out r) + B_l y_l(k_out r)) Y_l0(theta), B_l = i A_l; inside,
sum_l C_l j_l(k_in r) Y_l0(theta).  A_l and C_l follow from continuity of the
fluence and of the normal flux at r = a.  The semi-infinite and slab versions
add image sources (extrapolated boundary z_b = 2D(1+R)/(1-R), source depth
z_0 = 1/mu_s') and the first-order images of the sphere.

Pinned by tests/golden/sphdiffsemiinf.npz (the reference's
examples/meshtest/sphdiffsemiinf.mat).  `point_semi_infinite` is the
homogeneous semi-infinite medium in closed form (the same image sources with
no sphere), equal to `semi_infinite` with a sphere of the background's
properties.
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np
from scipy.special import eval_legendre, spherical_jn, spherical_yn


@dataclass(frozen=True)
class SphereCfg:
    """cfg of the reference toolbox; defaults as matlab/sphdiffusionslab.m:45-56."""
    v: float = 299792458000.0   # speed of light, mm/s
    a: float = 10.0             # sphere radius, mm
    omua: float = 0.002         # background mua, 1/mm
    omusp: float = 0.990        # background mus', 1/mm
    imua: float = 0.050         # sphere mua
    imusp: float = 0.500        # sphere mus'
    src: tuple = (30.0, np.pi, 0.0)   # source (R, theta, phi) about the sphere centre
    maxl: int = 20
    omega: float = 0.0

    @property
    def Din(self):
        return self.v / (3 * self.imusp)

    @property
    def Dout(self):
        return self.v / (3 * self.omusp)

    @property
    def kin(self):
        return np.sqrt(complex(-self.v * self.imua, self.omega) / self.Din)

    @property
    def kout(self):
        return np.sqrt(complex(-self.v * self.omua, self.omega) / self.Dout)


def _h1(n, z, derivative=False):
    return spherical_jn(n, z, derivative) + 1j * spherical_yn(n, z, derivative)


def _y_l0(l, theta):
    """Spherical harmonic Y_l^0(theta)."""
    return np.sqrt((2 * l + 1) / (4 * np.pi)) * eval_legendre(l, np.cos(theta))


def _axial(cfg):
    th = cfg.src[1]
    if not (th == 0.0 or th == np.pi):
        raise ValueError("only sources on the sphere's axis (theta = 0 or pi) are restated")


def _coeff_common(l, cfg):
    x, y = cfg.kout * cfg.a, cfg.kin * cfg.a
    pre = -1j * cfg.v * cfg.kout / cfg.Dout * _h1(l, cfg.kout * cfg.src[0]) * np.conj(_y_l0(l, cfg.src[1]))
    den = (cfg.Dout * x * _h1(l, x, True) * spherical_jn(l, y)
           - cfg.Din * y * _h1(l, x) * spherical_jn(l, y, True))
    return x, y, pre, den


def acoeff(l, cfg):
    """A_l (m = 0): matlab/sphdiffAcoeff.m."""
    x, y, pre, den = _coeff_common(l, cfg)
    num = (cfg.Dout * x * spherical_jn(l, x, True) * spherical_jn(l, y)
           - cfg.Din * y * spherical_jn(l, x) * spherical_jn(l, y, True))
    return pre * num / den


def ccoeff(l, cfg):
    """C_l (m = 0): matlab/sphdiffCcoeff.m."""
    x, y, pre, den = _coeff_common(l, cfg)
    num = (cfg.Dout * x * _h1(l, x) * spherical_jn(l, x, True)
           - cfg.Dout * x * _h1(l, x, True) * spherical_jn(l, x))
    return pre * num / den


def _sph(x, y, z):
    """(r, theta from +z, phi) of Cartesian points."""
    r = np.sqrt(x * x + y * y + z * z)
    theta = np.arccos(np.clip(np.divide(z, r, out=np.ones_like(r), where=r > 0), -1.0, 1.0))
    return r, theta, np.arctan2(y, x)


def incident(x, y, z, cfg):
    """matlab/sphdiffincident.m: the source's free-space Green's function."""
    R, th, ph = cfg.src
    xs, ys, zs = R * np.sin(th) * np.cos(ph), R * np.sin(th) * np.sin(ph), R * np.cos(th)
    d = np.sqrt((x - xs) ** 2 + (y - ys) ** 2 + (z - zs) ** 2)
    return cfg.v / (4 * np.pi * cfg.Dout * d) * np.exp(1j * cfg.kout * d)


def scatter(r, theta, cfg):
    """matlab/sphdiffscatter.m (m = 0 terms)."""
    res = np.zeros(r.shape, complex)
    for l in range(cfg.maxl + 1):
        a = acoeff(l, cfg)
        res += (a * spherical_jn(l, cfg.kout * r) + 1j * a * spherical_yn(l, cfg.kout * r)) * _y_l0(l, theta)
    return res


def interior(r, theta, cfg):
    """matlab/sphdiffinterior.m (m = 0 terms)."""
    res = np.zeros(r.shape, complex)
    for l in range(cfg.maxl + 1):
        res += ccoeff(l, cfg) * spherical_jn(l, cfg.kin * r) * _y_l0(l, theta)
    return res


def infinite(x, y, z, cfg):
    """matlab/sphdiffusioninfinite.m on points (x, y, z) about the sphere centre."""
    _axial(cfg)
    r, th, _ = _sph(x, y, z)
    res = np.zeros(r.shape, complex)
    out = r > cfg.a
    res[out] = incident(x[out], y[out], z[out], cfg) + scatter(r[out], th[out], cfg)
    res[~out] = interior(r[~out], th[~out], cfg)
    return res


def scatter_only(x, y, z, cfg):
    """matlab/sphdiffusionscatteronly.m."""
    _axial(cfg)
    r, th, _ = _sph(x, y, z)
    res = np.zeros(r.shape, complex)
    out = r > cfg.a
    res[out] = scatter(r[out], th[out], cfg)
    return res


def _zb_z0(reff, cfg):
    D = 1 / (3 * (cfg.omua + cfg.omusp))
    return (1 + reff) / (1 - reff) * 2 * D, 1 / (cfg.omusp + cfg.omua)


def semi_infinite(reff, x, y, z, cfg):
    """matlab/sphdiffusionsemi.m: the surface is the plane through the source
    (at depth src[0] below the sphere centre), extrapolated by z_b."""
    zb, z0 = _zb_z0(reff, cfg)
    s0 = cfg.src
    res = infinite(x, y, z, replace(cfg, src=(s0[0] - z0, s0[1], s0[2])))                  # S1,O1
    res -= infinite(x, y, z, replace(cfg, src=(s0[0] + z0 + 2 * zb, np.pi, s0[2])))         # S2,O1
    out = _sph(x, y, z)[0] > cfg.a
    zs = z + 2 * (s0[0] + zb)
    res[out] += scatter_only(x, y, zs, replace(cfg, src=(s0[0] + z0 + 2 * zb, 0.0, s0[2])))[out]  # S1,O2
    res[out] -= scatter_only(x, y, zs, replace(cfg, src=(s0[0] - z0, 0.0, s0[2])))[out]           # S2,O2
    return res


def slab(reff1, reff2, h, x, y, z, cfg=SphereCfg()):
    """matlab/sphdiffusionslab.m: a slab of thickness h (source surface at
    depth src[0] below the sphere centre, the other surface h below it)."""
    zb, z0 = _zb_z0(reff2, cfg)
    s0 = cfg.src
    res = semi_infinite(reff1, x, y, z, cfg)
    res -= infinite(x, y, z, replace(cfg, src=(2 * h - s0[0] + 2 * zb - z0, np.pi - s0[1], s0[2])))
    res += infinite(x, y, z, replace(cfg, src=(2 * h - s0[0] + 2 * zb - z0 + 2 * (z0 + zb), np.pi - s0[1], s0[2])))
    out = _sph(x, y, z)[0] > cfg.a
    zs = z - 2 * (h - s0[0] + zb)
    res[out] += scatter_only(x, y, zs, replace(cfg, src=(2 * h - s0[0] - z0, s0[1], s0[2])))[out]
    res[out] -= scatter_only(x, y, zs, replace(cfg, src=(2 * h - s0[0] + 2 * zb + z0, s0[1], s0[2])))[out]
    res[out] -= scatter_only(x, y, zs, replace(cfg, src=(s0[0] - z0, np.pi - s0[1], s0[2])))[out]
    res[out] += scatter_only(x, y, zs, replace(cfg, src=(s0[0] + 2 * zb + z0, np.pi - s0[1], s0[2])))[out]
    return res


def point_semi_infinite(reff, mua, musp, x, y, depth, v=299792458000.0):
    """Continuous-wave fluence of a unit pencil source entering a homogeneous
    semi-infinite medium at the origin, at points (x, y) and `depth` below the
    surface: the source moved to depth z0 = 1/(mua + mus') and its image at
    -(z0 + 2 z_b), z_b = 2D(1+R)/(1-R), D = 1/(3(mua + mus')), as
    matlab/sphdiffusionsemi.m builds them, each with the Green's function of
    matlab/sphdiffincident.m (v/(4 pi D' d) exp(-mu_eff d), D' = v/(3 mus'))."""
    D = 1.0 / (3.0 * (mua + musp))
    zb = (1.0 + reff) / (1.0 - reff) * 2.0 * D
    z0 = 1.0 / (musp + mua)
    dout = v / (3.0 * musp)
    mueff = np.sqrt(v * mua / dout)
    r1 = np.sqrt(x * x + y * y + (depth - z0) ** 2)
    r2 = np.sqrt(x * x + y * y + (depth + z0 + 2.0 * zb) ** 2)
    return v / (4.0 * np.pi * dout) * (np.exp(-mueff * r1) / r1 - np.exp(-mueff * r2) / r2)
