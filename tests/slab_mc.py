"""An independent Monte Carlo of a laterally infinite layered slab (numpy),
written from the standard layered-medium algorithm (optical depth spent layer
by layer, Fresnel reflection at every index step with the z normal,
Henyey-Greenstein scattering, roulette), to check the voxel-boundary
stepping of the oracle and of the engine on the same physics.  Weights are
real numbers here; the engine's are fixed-point integers."""
from __future__ import annotations

import numpy as np


def fresnel(n1: float, n2: float, cos_i: np.ndarray) -> np.ndarray:
    """Unpolarised Fresnel reflectance (1 beyond the critical angle)."""
    cos_i = np.clip(cos_i, 0.0, 1.0)
    sin_t = n1 / n2 * np.sqrt(np.maximum(0.0, 1.0 - cos_i * cos_i))
    tir = sin_t >= 1.0
    cos_t = np.sqrt(np.maximum(0.0, 1.0 - sin_t * sin_t))
    with np.errstate(invalid="ignore", divide="ignore"):
        rs = ((n1 * cos_i - n2 * cos_t) / (n1 * cos_i + n2 * cos_t)) ** 2
        rp = ((n1 * cos_t - n2 * cos_i) / (n1 * cos_t + n2 * cos_i)) ** 2
    r = 0.5 * (rs + rp)
    r = np.where(cos_i >= 1.0, ((n1 - n2) / (n1 + n2)) ** 2, r)
    return np.where(tir, 1.0, r)


def run(layers, n_above: float, n_below: float, photons: int, seed: int):
    """layers: [(thickness, mua, mus, g, n), ...] top to bottom.  Returns the
    fractions of the launched weight (R, T, A) for a collimated beam."""
    rng = np.random.default_rng(seed)
    z_top = np.cumsum([0.0] + [l[0] for l in layers])[:-1]
    z_bot = np.cumsum([l[0] for l in layers])
    mua = np.array([l[1] for l in layers])
    mut = np.array([l[1] + l[2] for l in layers])
    g = np.array([l[3] for l in layers])
    n = np.array([l[4] for l in layers])
    nl = len(layers)
    r_sp = ((n_above - n[0]) / (n_above + n[0])) ** 2
    w0 = 1.0 - r_sp
    N = photons
    z = np.zeros(N)
    ux = np.zeros(N)
    uy = np.zeros(N)
    uz = np.ones(N)
    w = np.full(N, w0)
    lay = np.zeros(N, dtype=int)
    alive = np.ones(N, dtype=bool)
    R = T = A = 0.0
    while alive.any():
        idx = np.nonzero(alive)[0]
        tau = -np.log(1.0 - rng.random(idx.size))
        act = idx.copy()
        # spend the optical depth layer by layer
        while act.size:
            L = lay[act]
            dz = uz[act]
            db = np.where(dz > 0, (z_bot[L] - z[act]) / np.where(dz > 0, dz, 1.0),
                          np.where(dz < 0, (z_top[L] - z[act]) / np.where(dz < 0, dz, 1.0), np.inf))
            s = tau / mut[L]
            hit = s <= db
            # interactions
            ih = act[hit]
            z[ih] += uz[ih] * s[hit]
            # boundary crossings
            ib = act[~hit]
            tb = tau[~hit] - db[~hit] * mut[L[~hit]]
            z[ib] += uz[ib] * db[~hit]
            Lb = lay[ib]
            up = uz[ib] < 0
            nxt = Lb + np.where(up, -1, 1)
            n1 = n[Lb]
            n2 = np.where(nxt < 0, n_above, np.where(nxt >= nl, n_below, n[np.clip(nxt, 0, nl - 1)]))
            cos_i = np.abs(uz[ib])
            refl = np.zeros(ib.size, dtype=bool)
            same = n1 == n2
            for a in np.unique(n1[~same]):
                for b2 in np.unique(n2[~same]):
                    m = (~same) & (n1 == a) & (n2 == b2)
                    if m.any():
                        refl[m] = rng.random(m.sum()) <= fresnel(a, b2, cos_i[m])
            # reflected: mirror uz, keep the remaining depth
            uz[ib[refl]] *= -1.0
            # transmitted: refract, change layer or leave
            tr = ~refl
            it_ = ib[tr]
            ratio = (n1 / n2)[tr]
            uxt, uyt = ux[it_] * ratio, uy[it_] * ratio
            uzt = np.sign(uz[it_]) * np.sqrt(np.maximum(0.0, 1.0 - uxt * uxt - uyt * uyt))
            ux[it_], uy[it_], uz[it_] = uxt, uyt, uzt
            nt = nxt[tr]
            out_top = nt < 0
            out_bot = nt >= nl
            R += w[it_[out_top]].sum()
            T += w[it_[out_bot]].sum()
            alive[it_[out_top | out_bot]] = False
            w[it_[out_top | out_bot]] = 0.0
            stay = ~(out_top | out_bot)
            lay[it_[stay]] = nt[stay]
            # continue the photons still travelling
            cont = np.concatenate([ib[refl], it_[stay]])
            tau_c = np.concatenate([tb[refl], tb[tr][stay]])
            act, tau = cont, tau_c
            # interactions of this round: absorb and scatter
            if ih.size:
                Li = lay[ih]
                dw = w[ih] * mua[Li] / mut[Li]
                A += dw.sum()
                w[ih] -= dw
                gg = g[Li]
                xi = rng.random(ih.size)
                with np.errstate(invalid="ignore", divide="ignore"):
                    tmp = (1 - gg * gg) / (1 - gg + 2 * gg * xi)
                    ct = np.where(gg != 0, (1 + gg * gg - tmp * tmp) / (2 * gg), 2 * xi - 1)
                ct = np.clip(ct, -1.0, 1.0)
                st = np.sqrt(1 - ct * ct)
                ph = 2 * np.pi * rng.random(ih.size)
                cp, sp = np.cos(ph), np.sin(ph)
                x0, y0, z0 = ux[ih], uy[ih], uz[ih]
                den = np.sqrt(np.maximum(1e-30, 1 - z0 * z0))
                vert = np.abs(z0) > 0.99999
                nxv = np.where(vert, st * cp, st * (x0 * z0 * cp - y0 * sp) / den + x0 * ct)
                nyv = np.where(vert, st * sp, st * (y0 * z0 * cp + x0 * sp) / den + y0 * ct)
                nzv = np.where(vert, np.sign(z0) * ct, -st * cp * den + z0 * ct)
                nrm = np.sqrt(nxv * nxv + nyv * nyv + nzv * nzv)
                ux[ih], uy[ih], uz[ih] = nxv / nrm, nyv / nrm, nzv / nrm
                # roulette
                low = w[ih] < 1e-4 * w0
                il = ih[low]
                live = rng.random(il.size) < 0.1
                w[il[live]] /= 0.1
                w[il[~live]] = 0.0
                alive[il[~live]] = False
                ih = ih[:0]
    return R / (photons * w0), T / (photons * w0), A / (photons * w0)
