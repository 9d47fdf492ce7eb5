"""FP64 restatement of the reference's canonical thermodynamics (TEST INFRASTRUCTURE ONLY).

Follows Thermodynamics::calculate_thermodynamics (src/Thermodynamics/thermodynamics.hpp:
158-236 with TRAPEZOIDAL_RULE, 238-297 without): for T = Tmin + i (Tmax - Tmin) / nT,
x_b = ln g_b - E_b / T, m = max_b x_b, w_b = exp(x_b - m) (halved at the two end bins under
the trapezoidal rule), Z = sum w; F = -T (m + ln Z) / N, U = sum E w / (N Z),
U2 = sum E^2 w / (N^2 Z), S = sum ln g w / (N Z), C = N (U2 - U^2) / T^2, observables
sum O w / Z, and the counts column averaged over the bins.  Rows are
[F, U, U2, S, C, observables...] as the reference's canonical_observables.
The nonlinear observables follow order_parameter_cumulants.hpp:17-48 and
calculate_nonlinear_observables (ising2d_observables.hpp:166-198,
ashkin_teller2d_observables.hpp:243-282), without correlation lengths.
"""
from __future__ import annotations

import numpy as np


def temperatures(Tmin: float, Tmax: float, nT: int) -> np.ndarray:
    dT = (Tmax - Tmin) / nT
    return Tmin + dT * np.arange(nT, dtype=np.float64)


def thermodynamics(E, lng, obs, N, Tmin, Tmax, nT, counts_col=None, trapezoid=True, chunk=512):
    E = np.asarray(E, dtype=np.float64)
    lng = np.asarray(lng, dtype=np.float64)
    nb = E.size
    K = 0 if obs is None else obs.shape[1]
    T = temperatures(Tmin, Tmax, nT)
    f = np.ones(nb)
    if trapezoid:
        f[0] = f[-1] = 0.5
    out = np.zeros((nT, 5 + K))
    for a in range(0, nT, chunk):
        t = T[a:a + chunk, None]
        x = lng[None, :] - E[None, :] / t
        m = x.max(axis=1, keepdims=True)
        w = np.exp(x - m) * f[None, :]
        Z = w.sum(axis=1)
        U = (w * E).sum(axis=1) / (N * Z)
        U2 = (w * E * E).sum(axis=1) / (N * N * Z)
        out[a:a + chunk, 0] = -t[:, 0] * (m[:, 0] + np.log(Z)) / N
        out[a:a + chunk, 1] = U
        out[a:a + chunk, 2] = U2
        out[a:a + chunk, 3] = (w * lng).sum(axis=1) / (N * Z)
        out[a:a + chunk, 4] = N * (U2 - U * U) / (t[:, 0] ** 2)
        for k in range(K):
            if k == counts_col:
                out[a:a + chunk, 5 + k] = obs[:, k].sum() / nb
            else:
                out[a:a + chunk, 5 + k] = (w * obs[None, :, k]).sum(axis=1) / Z
    return T, out


def susceptibility(m2, m, T, N):
    return N * (m2 - m * m) / T


def binder(m4, m2):
    return 1.0 - (m4 / (m2 * m2)) / 3.0


def binder_two_component(m4, m2):
    return 2.0 * (1.0 - 0.5 * (m4 / (m2 * m2)))


def correlation_length_over_L(G0, Gq, N):
    """calculate_correlation_length(G0, Gq, L) / L with L = (size_t) sqrt(N)
    (order_parameter_cumulants.hpp:52-59, ising2d_observables.hpp:180-190)."""
    L = float(int(np.sqrt(N)))
    G0, Gq = np.asarray(G0, dtype=np.float64), np.asarray(Gq, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        x = (L / (2.0 * np.arccos(-1.0))) * np.sqrt((G0 - Gq) / Gq)
    x = np.where(Gq == 0.0, np.finfo(np.float64).max, x)
    return x / L


def nonlinear(model: int, rows, T, N, correlators: bool = False):
    """Ising: [susceptibility, Binder cumulant]; Ashkin-Teller: sigma, tau, Baxter
    (susceptibility, Binder cumulant) then phi (susceptibility, two-component cumulant).
    With correlators (CORRELATION_LENGTHS layout: G(q_min) after each group of three moments)
    each pair is followed by the correlation length over L."""
    o = rows[:, 5:]
    if correlators:
        if model == 0:
            return np.stack([susceptibility(o[:, 1], o[:, 0], T, N), binder(o[:, 2], o[:, 1]),
                             correlation_length_over_L(o[:, 1], o[:, 3], N)], axis=1)
        cols = []
        for base in (0, 4, 12):     # sigma, tau, Baxter
            g = o[:, base:base + 4]
            cols += [susceptibility(g[:, 1], g[:, 0], T, N), binder(g[:, 2], g[:, 1]),
                     correlation_length_over_L(g[:, 1], g[:, 3], N)]
        g = o[:, 8:12]              # phi
        cols += [susceptibility(g[:, 1], g[:, 0], T, N), binder_two_component(g[:, 2], g[:, 1]),
                 correlation_length_over_L(g[:, 1], g[:, 3], N)]
        return np.stack(cols, axis=1)
    if model == 0:
        return np.stack([susceptibility(o[:, 1], o[:, 0], T, N), binder(o[:, 2], o[:, 1])], axis=1)
    cols = []
    for base in (0, 3, 9):          # sigma, tau, Baxter
        cols += [susceptibility(o[:, base + 1], o[:, base], T, N), binder(o[:, base + 2], o[:, base + 1])]
    cols += [susceptibility(o[:, 7], o[:, 6], T, N), binder_two_component(o[:, 8], o[:, 7])]
    return np.stack(cols, axis=1)
