"""Continuous spectral densities and their discretisation into harmonic modes.

Host-side preprocessing of the spin-boson driver (src/spin_boson.cpp:156-380): the
reference reads a bath from its input file, finds the frequency window to keep, and
discretises the window by the Gauss quadrature rule of the bath's measure; mode k gets
frequency w_k (a node) and coupling g_k = sqrt(W_k / pi) (W_k its weight).

Spectral densities restate src/bath/bath_types/{exponential,sudden,gaussian,debye,
jacobi_cutoff}.hpp: J(w) is extended to negative frequencies as an odd function and, at
inverse temperature beta, the measure discretised is 0.5 (S(w) + J(w)) = J(w) / (1 -
exp(-beta w)) on [w_min, w_max] with w_min < 0 (negative-frequency modes stand in for
the thermal bath, spin_boson.cpp:327-343); at zero temperature it is J(w) on [0, w_max]
(spin_boson.cpp:345-355).

The reference builds the quadrature with the orthopol library of its utils_cpp
submodule (github.com/llindoy/utils_cpp, not vendored with the reference): Jacobi
polynomials on the window, the orthogonal polynomials of the bath measure from them
(``nonclassical_polynomial``) and the Golub-Welsch nodes and weights.  The Gauss rule of
a positive measure is unique, so this module reaches the same nodes and weights by a
different, published route: the measure is discretised by a composite Gauss-Legendre /
Gauss-Jacobi rule fine enough to integrate every polynomial of degree 2N exactly to
double precision, the recurrence coefficients of the discrete measure come from the
Lanczos process with full reorthogonalisation (the discretised Stieltjes procedure,
W. Gautschi, "Orthogonal Polynomials: Computation and Approximation", OUP 2004, sec.
2.2), and the nodes and weights from the eigen-decomposition of the Jacobi matrix
(G. H. Golub and J. H. Welsch, Math. Comp. 23, 221 (1969)).  The reference's
``moment scaling``, ``jacobi alpha`` and ``jacobi beta`` inputs only condition its
modified-moment algorithm and leave the rule unchanged; they are accepted and ignored.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np


def _norm_key(k: str) -> str:
    """Input keys are matched with whitespace removed and lower-cased
    (io::remove_whitespace_and_to_lower, used by every IOWRAPPER::load of the driver)."""
    return "".join(k.split()).lower()


def normalise_keys(obj):
    """Dictionary with normalised keys (recursively); later duplicates win, as in a JSON
    object read member by member."""
    if isinstance(obj, dict):
        return {_norm_key(k): normalise_keys(v) for k, v in obj.items()}
    if isinstance(obj, list):
        return [normalise_keys(v) for v in obj]
    return obj


class SpectralDensity:
    """Base of the continuous baths (src/bath/bath_types/bath.hpp:19-321,
    continuous_bath :323-366).  ``beta`` is None at zero temperature."""

    type_name = ""

    def __init__(self, beta: Optional[float] = None):
        self.beta = beta

    # -- to be provided by each bath ------------------------------------------------------
    def J(self, w):
        raise NotImplementedError

    def density(self, w):
        """``density_of_frequencies`` (used to place the frequency window)."""
        raise NotImplementedError

    def upper_bound(self, tol: float) -> float:
        raise NotImplementedError

    def breakpoints(self) -> List[Tuple[float, float, float]]:
        """Points where the measure is not analytic: (w, exponent on the left side,
        exponent on the right side) of the local power law |w - w0|^e (0 for a jump or a
        plain breakpoint)."""
        return []

    # -- shared ----------------------------------------------------------------------------
    @property
    def nonzero_temperature(self) -> bool:
        return self.beta is not None

    def S(self, w):
        """Noise power spectrum J(w) coth(beta w / 2) (J(w) at zero temperature)."""
        w = np.asarray(w, dtype=np.float64)
        if not self.nonzero_temperature:
            return self.J(w)
        return self.J(w) / np.tanh(0.5 * self.beta * w)

    def measure(self, w):
        """The measure that is discretised: 0.5 (S + J) = J / (1 - exp(-beta w)) at finite
        temperature (spin_boson.cpp:340), J at zero temperature (:352)."""
        w = np.asarray(w, dtype=np.float64)
        if not self.nonzero_temperature:
            return self.J(w)
        with np.errstate(divide="ignore", invalid="ignore"):
            out = self.J(w) / (-np.expm1(-self.beta * w))
        # w = 0 exactly: the limit J(w) / (beta w); only reached by a caller, never by a node
        z = w == 0.0
        if np.any(z):
            h = 1e-300
            out = np.where(z, self.J(np.full_like(w, h)) / (self.beta * h), out)
        return out

    def frequency_bounds(self, tol: float, thermofield: bool = True) -> Tuple[float, float]:
        """``frequency_bounds(tol, quad, use_thermofield)``: the window holding all but a
        fraction ``tol`` of the bath (exponential.hpp:104-131 and the same member of
        every bath type).  With ``thermofield`` at finite temperature the lower bound is
        the negative frequency where the Boltzmann-weighted density exp(-beta w) rho(w)
        reaches 1 - tol of its integral over [0, w_max]."""
        hi = float(self.upper_bound(tol))
        lo = 0.0
        if thermofield and self.nonzero_temperature:
            f = lambda x: float(self.density(np.float64(x))) * math.exp(-self.beta * x)
            total = _integrate(f, 0.0, hi)
            lo = -_max_frequency(f, total * (1.0 - tol), hi / 2.0)
        return lo, hi


def _integrate(f, a: float, b: float) -> float:
    from scipy.integrate import quad
    val, _ = quad(f, a, b, epsabs=0.0, epsrel=1e-13, limit=400)
    return float(val)


def _max_frequency(rho, target: float, w0: float) -> float:
    """The w with int_0^w rho = target (discretisation_utilities.hpp:8-17 solves the same
    equation by damped Newton steps; here by bracketing and Brent's method)."""
    from scipy.optimize import brentq
    F = lambda w: _integrate(rho, 0.0, w) - target
    hi = max(w0, 1e-12)
    for _ in range(200):
        if F(hi) > 0.0:
            break
        hi *= 2.0
    else:
        raise ValueError("failed to bracket the maximum frequency")
    return float(brentq(F, 0.0, hi, xtol=1e-14 * hi, rtol=1e-15, maxiter=500))


class Exponential(SpectralDensity):
    """J(w) = pi alpha / 2 wc (|w| / wc)^s exp(-|w| / wc) sign(w)
    (src/bath/bath_types/exponential.hpp:36-39, density :93-97, bounds :104-131)."""

    type_name = "exponential"

    def __init__(self, alpha: float, wc: float, s: float = 1.0, beta: Optional[float] = None):
        super().__init__(beta)
        self.alpha, self.wc, self.s = float(alpha), float(wc), float(s)

    def J(self, w):
        w = np.asarray(w, dtype=np.float64)
        a = np.abs(w)
        return math.pi * self.alpha / 2.0 * self.wc * (a / self.wc) ** self.s * np.exp(-a / self.wc) * np.where(
            w < 0, -1.0, 1.0)

    def density(self, w):
        w = np.asarray(w, dtype=np.float64)
        if self.s < 1:
            return self.J(w)
        return math.pi / 2.0 * self.alpha * (np.abs(w) / self.wc) ** (self.s - 1.0) * np.exp(-np.abs(w) / self.wc)

    def upper_bound(self, tol):
        if self.s > 1:
            lam = math.gamma(self.s) * self.alpha * self.wc / 2.0
            f = lambda x: float(self.density(np.float64(x)))
            return _max_frequency(f, lam * math.pi * (1.0 - tol), self.wc * math.log(1.0 / tol))
        return self.wc * math.log(1.0 / tol)

    def breakpoints(self):
        return [(0.0, *_zero_exponents(self.s, self.nonzero_temperature))]


class Sudden(SpectralDensity):
    """J(w) = pi alpha Gamma(s+1) / 2 wc (|w| / wc)^s sign(w) for |w| < wc, else 0
    (src/bath/bath_types/sudden.hpp:37-40, density :66-70, bounds :76-93)."""

    type_name = "sudden"

    def __init__(self, alpha: float, wc: float, s: float = 1.0, beta: Optional[float] = None):
        super().__init__(beta)
        self.alpha, self.wc, self.s = float(alpha), float(wc), float(s)

    def _pref(self):
        return math.pi * self.alpha * math.gamma(self.s + 1.0) / 2.0

    def J(self, w):
        w = np.asarray(w, dtype=np.float64)
        a = np.abs(w)
        return np.where(a < self.wc, self._pref() * self.wc * (a / self.wc) ** self.s, 0.0) * np.where(w < 0, -1.0, 1.0)

    def density(self, w):
        w = np.asarray(w, dtype=np.float64)
        if self.s < 1:
            return self.J(w)
        a = np.abs(w)
        return np.where(a < self.wc, self._pref() * (a / self.wc) ** (self.s - 1.0), 0.0) * np.where(w < 0, -1.0, 1.0)

    def upper_bound(self, tol):
        return self.wc

    def breakpoints(self):
        return [(0.0, *_zero_exponents(self.s, self.nonzero_temperature)), (self.wc, 0.0, 0.0), (-self.wc, 0.0, 0.0)]


class Gaussian(SpectralDensity):
    """J(w) = sqrt(pi/2) alpha w exp(-w^2 / (2 wc^2))
    (src/bath/bath_types/gaussian.hpp:36-39, density :65-68, bounds :74-93)."""

    type_name = "gaussian"

    def __init__(self, alpha: float, wc: float, beta: Optional[float] = None):
        super().__init__(beta)
        self.alpha, self.wc = float(alpha), float(wc)
        self.s = 1.0

    def J(self, w):
        w = np.asarray(w, dtype=np.float64)
        return math.sqrt(math.pi / 2.0) * self.alpha * w * np.exp(-w * w / (self.wc * self.wc * 2.0))

    def density(self, w):
        w = np.asarray(w, dtype=np.float64)
        return math.sqrt(math.pi / 2.0) * self.alpha * np.exp(-w * w / (self.wc * self.wc * 2.0))

    def upper_bound(self, tol):
        lam = self.alpha * self.wc / 2.0
        f = lambda x: float(self.density(np.float64(x)))
        return _max_frequency(f, lam * math.pi * (1.0 - tol), self.wc * math.log(1.0 / tol))


class Debye(SpectralDensity):
    """J(w) = alpha wc^2 w / (w^2 + wc^2), alpha = 2 lambda / wc when the reorganisation
    energy lambda is given (src/bath/bath_types/debye.hpp:35-38, density :66, bounds
    :69-85, load :108-130)."""

    type_name = "debye"

    def __init__(self, alpha: float, wc: float, beta: Optional[float] = None):
        super().__init__(beta)
        self.alpha, self.wc = float(alpha), float(wc)
        self.s = 1.0

    def J(self, w):
        w = np.asarray(w, dtype=np.float64)
        return self.alpha * self.wc * self.wc * w / (w * w + self.wc * self.wc)

    def density(self, w):
        w = np.asarray(w, dtype=np.float64)
        return self.alpha * self.wc * self.wc / (2.0 * (w * w + self.wc * self.wc))

    def upper_bound(self, tol):
        return self.wc * math.tan((1.0 - tol) * math.pi / 2.0)


class JacobiCutoff(SpectralDensity):
    """J(w) = pi alpha Gamma(s+q+1) / (2 Gamma(q+1)) wc (|w|/wc)^s (1 - |w|/wc)^q sign(w)
    for |w| < wc (src/bath/bath_types/jacobi_cutoff.hpp:39-42, density :70-74, bounds
    :80-97)."""

    type_name = "jacobi"

    def __init__(self, alpha: float, wc: float, s: float, q: float, beta: Optional[float] = None):
        super().__init__(beta)
        self.alpha, self.wc, self.s, self.q = float(alpha), float(wc), float(s), float(q)

    def _pref(self):
        return math.pi * self.alpha * math.exp(math.lgamma(self.s + self.q + 1.0) - math.lgamma(self.q + 1.0)) / 2.0

    def J(self, w):
        w = np.asarray(w, dtype=np.float64)
        a = np.abs(w)
        inside = a < self.wc
        ac = np.where(inside, a, 0.0)
        val = self._pref() * self.wc * (ac / self.wc) ** self.s * (1.0 - ac / self.wc) ** self.q
        return np.where(inside, val, 0.0) * np.where(w < 0, -1.0, 1.0)

    def density(self, w):
        w = np.asarray(w, dtype=np.float64)
        if self.s < 1:
            return self.J(w)
        a = np.abs(w)
        inside = a < self.wc
        ac = np.where(inside, a, 0.0)
        val = self._pref() * (ac / self.wc) ** (self.s - 1.0) * (1.0 - ac / self.wc) ** self.q
        return np.where(inside, val, 0.0) * np.where(w < 0, -1.0, 1.0)

    def upper_bound(self, tol):
        return self.wc

    def breakpoints(self):
        return [(0.0, *_zero_exponents(self.s, self.nonzero_temperature)), (self.wc, self.q, 0.0),
                (-self.wc, 0.0, self.q)]


def _zero_exponents(s: float, finite_t: bool) -> Tuple[float, float]:
    """Local power of the measure at w = 0: |w|^s at zero temperature, |w|^(s-1) at finite
    temperature (J / (1 - exp(-beta w)) ~ J / (beta w)); integer powers are analytic."""
    e = s - 1.0 if finite_t else s
    if abs(e - round(e)) < 1e-14 and e >= 0:
        e = 0.0
    return e, e


_BATHS = {"exponential": Exponential, "sudden": Sudden, "gaussian": Gaussian, "debye": Debye, "jacobi": JacobiCutoff}


def load_bath(obj: Dict) -> SpectralDensity:
    """The bath of an input file (io::factory<continuous_bath>::create, spin_boson.cpp:196;
    abstract_bath::load, bath.hpp:274-318): ``type`` names the bath; ``beta`` or a
    nonzero ``t`` selects a finite temperature."""
    o = normalise_keys(obj)
    if "type" not in o:
        raise ValueError("bath: missing type")
    name = _norm_key(str(o["type"]))
    beta = None
    if "beta" in o:
        beta = float(o["beta"])
    elif "t" in o:
        T = float(o["t"])
        if T < 0:
            raise ValueError("bath: invalid temperature")
        if abs(T) > 1e-14:
            beta = 1.0 / T

    def need(k):
        if k not in o:
            raise ValueError(f"bath {name}: missing {k}")
        v = float(o[k])
        return v

    if name == "exponential":
        b = Exponential(need("alpha"), need("wc"), need("s"), beta)
    elif name == "sudden":
        b = Sudden(need("alpha"), need("wc"), need("s"), beta)
    elif name == "gaussian":
        b = Gaussian(need("alpha"), need("wc"), beta)
    elif name == "debye":
        wc = need("wc")
        if "alpha" in o:
            alpha = float(o["alpha"])
        elif "lambda" in o:
            alpha = 2.0 * float(o["lambda"]) / wc
        else:
            raise ValueError("bath debye: missing alpha or lambda")
        b = Debye(alpha, wc, beta)
    elif name == "jacobi":
        b = JacobiCutoff(need("alpha"), need("wc"), need("s"), need("q"), beta)
    else:
        raise ValueError(f"unknown bath type {o['type']!r}; known: {sorted(_BATHS)}")
    if getattr(b, "wc", 0.0) < 0 or getattr(b, "alpha", 0.0) < 0 or getattr(b, "s", 0.0) < 0:
        raise ValueError("bath: negative parameter")
    return b


# --------------------------------------------------------------------------------------
# Gauss quadrature of the bath measure
# --------------------------------------------------------------------------------------

_PANEL_POINTS = 32


def _panel_edges(lo: float, hi: float, N: int, points: Sequence[Tuple[float, float, float]]) -> np.ndarray:
    """Panel edges: Chebyshev-spaced over [lo, hi] (the oscillation of a degree-2N
    polynomial concentrates towards the ends), the breakpoints of the measure, and
    geometric grading towards w = 0 and every breakpoint (singular powers, the jump of a
    sudden cutoff, and the poles of the measure next to the real axis near w = 0)."""
    K = max(64, int(math.ceil(N / 3.0)) + 16)
    L = hi - lo
    edges = list(lo + 0.5 * L * (1.0 - np.cos(np.pi * np.arange(K + 1) / K)))
    centres = [0.0] + [p[0] for p in points]
    for c in centres:
        if not (lo <= c <= hi):
            continue
        edges.append(c)
        for k in range(1, 48):
            d = L * 2.0 ** (-k)
            for e in (c - d, c + d):
                if lo < e < hi:
                    edges.append(e)
    edges = np.unique(np.asarray(edges, dtype=np.float64))
    keep = [edges[0]]
    for e in edges[1:]:
        if e - keep[-1] > 1e-14 * L:
            keep.append(e)
    keep[-1] = hi
    keep[0] = lo
    return np.asarray(keep)


def _discretise_measure(bath: SpectralDensity, lo: float, hi: float, N: int) -> Tuple[np.ndarray, np.ndarray]:
    """Nodes x_j and positive weights v_j with sum_j v_j p(x_j) = int p dmu for every
    polynomial p of degree <= 2N (to double precision): Gauss-Legendre panels, and
    Gauss-Jacobi panels next to a singular power |w - w0|^e."""
    from scipy.special import roots_jacobi, roots_legendre
    pts = bath.breakpoints()
    sing = {}
    for (w0, el, er) in pts:
        sing[w0] = (el, er)
    edges = _panel_edges(lo, hi, N, pts)
    m = _PANEL_POINTS
    tl, wl = roots_legendre(m)
    xs, vs = [], []
    for a, b in zip(edges[:-1], edges[1:]):
        h = 0.5 * (b - a)
        e_left = sing.get(a, (0.0, 0.0))[1]
        e_right = sing.get(b, (0.0, 0.0))[0]
        if e_left != 0.0:
            # weight (1 + t)^e: x - a = h (1 + t)
            t, W = roots_jacobi(m, 0.0, e_left)
            x = a + h * (1.0 + t)
            v = W * h / (1.0 + t) ** e_left          # (x - a)^e = h^e (1 + t)^e
        elif e_right != 0.0:
            t, W = roots_jacobi(m, e_right, 0.0)
            x = a + h * (1.0 + t)
            v = W * h / (1.0 - t) ** e_right
        else:
            x = a + h * (1.0 + tl)
            v = wl * h
        xs.append(x)
        vs.append(v * bath.measure(x))
    x = np.concatenate(xs)
    v = np.concatenate(vs)
    if np.any(~np.isfinite(v)) or np.any(v < 0):
        raise ValueError("the bath measure is not positive and finite on the frequency window")
    return x, v


def gauss_rule(bath: SpectralDensity, lo: float, hi: float, N: int) -> Tuple[np.ndarray, np.ndarray]:
    """N-point Gauss rule of the bath measure on [lo, hi]: nodes ascending, weights W_k
    with sum_k W_k p(w_k) = int p dmu for deg p <= 2N - 1."""
    from scipy.linalg import eigh_tridiagonal
    x, v = _discretise_measure(bath, lo, hi, N)
    M = len(x)
    if N > M // 4:
        raise ValueError("too many modes for the discretisation")
    mu0 = float(np.sum(v))
    # Lanczos on diag(x) from sqrt(v): the recurrence coefficients of the discrete measure
    # (the discretised Stieltjes procedure), full reorthogonalisation, centred and scaled
    # abscissae for accuracy
    c = 0.5 * (hi + lo)
    s = 0.5 * (hi - lo)
    y = (x - c) / s
    Q = np.zeros((N, M))
    a = np.zeros(N)
    b = np.zeros(max(N - 1, 0))
    q = np.sqrt(v / mu0)
    q /= np.linalg.norm(q)
    Q[0] = q
    for k in range(N):
        z = y * Q[k]
        a[k] = float(Q[k] @ z)
        z -= a[k] * Q[k]
        if k > 0:
            z -= b[k - 1] * Q[k - 1]
        for _ in range(2):
            z -= Q[:k + 1].T @ (Q[:k + 1] @ z)
        if k + 1 < N:
            nb = float(np.linalg.norm(z))
            if not nb > 0:
                raise ValueError("Lanczos breakdown in the bath discretisation")
            b[k] = nb
            Q[k + 1] = z / nb
    theta, V = eigh_tridiagonal(a, b)
    nodes = c + s * theta
    weights = mu0 * V[0] ** 2
    return nodes, weights


def discretise(bath: SpectralDensity, N: int, lo: float, hi: float) -> Tuple[np.ndarray, np.ndarray]:
    """Frequencies and couplings of the N harmonic modes (spin_boson.cpp:357-381): the
    Gauss rule of the bath measure on [lo, hi] (lo = 0 at zero temperature), sorted by
    |w|, g_k = sqrt(W_k / pi)."""
    if not bath.nonzero_temperature:
        lo = 0.0
    nodes, weights = gauss_rule(bath, lo, hi, N)
    order = np.argsort(np.abs(nodes), kind="stable")
    w = nodes[order]
    g = np.sqrt(weights[order] / math.pi)
    return w, g
