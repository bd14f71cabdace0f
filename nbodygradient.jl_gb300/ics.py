"""Host-side initial conditions: orbital elements -> Cartesian state and jac_init.

Mirrors NbodyGradient.jl's InitialConditions API (the Julia caller of the
drop-in path computes these itself; this module lets Python callers build the
same State):
  Elements            src/ics/InitialConditions.jl:21-107
  ElementsIC          src/ics/InitialConditions.jl:142-241
  CartesianIC         src/ics/InitialConditions.jl:259-282
  hierarchy           src/ics/setup_hierarchy.jl:9-179
  init_nbody          src/ics/init_nbody.jl:13-162
  kepler_init         src/ics/kepler_init.jl:66-210
  ekepler             src/ics/kepler.jl:1-41
Arrays follow the reference's column-major conventions: elements is N x 7 with
rows (m, P, t0, e cos w, e sin w, I, Omega); x, v are 3 x N; jac_init is
7N x 7N with per-body columns (P, t0, ecosw, esinw, I, Omega, m).
"""
import math
import os

import numpy as np

GNEWT = 39.4845 / (365.242 * 365.242)  # src/NbodyGradient.jl:15
THIRD = 1.0 / 3.0


def _ieee_div(a, b):
    """a / b with IEEE results for a zero divisor (Julia's Float64 division; Python raises instead)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.float64(a) / np.float64(b))


def _ieee_rem(a, b):
    """Julia's a % b for Float64 (rem: the sign of a; NaN for b = 0, where math.fmod raises)."""
    with np.errstate(invalid="ignore"):
        return float(np.fmod(np.float64(a), np.float64(b)))


class Elements:
    """Orbital elements of one body (InitialConditions.jl:21-107), with the reference's three constructors:

      Elements(m, P, t0, ecosw, esinw, I, Omega)              e and w from ecosw, esinw; a = tp = 0; no checks
      Elements(m, P, t0, ecosw, esinw, I, Omega, a, e, w, tp)  the eleven fields as given
      Elements(m=..., P=..., ...)                              keywords, checked (the mass alone: a central body)

    Keywords may also be spelled as the reference spells them (ecosω, esinω, Ω, ω).
    """

    FIELDS = ("m", "P", "t0", "ecosw", "esinw", "I", "Omega")
    ALL_FIELDS = ("m", "P", "t0", "ecosw", "esinw", "I", "Omega", "a", "e", "w", "tp")
    _ALIASES = {"ecosω": "ecosw", "esinω": "esinw", "Ω": "Omega", "ω": "w"}

    def __init__(self, *args, **kw):
        if args and kw:
            raise TypeError("Elements takes positional fields or keywords, not both")
        if args:
            vals = [float(q) for q in args]
            if len(vals) == 7:  # InitialConditions.jl:38-42
                m, P, t0, ecosw, esinw, I, Omega = vals
                vals += [0.0, math.sqrt(ecosw * ecosw + esinw * esinw), math.atan2(esinw, ecosw), 0.0]
            elif len(vals) != 11:
                raise TypeError("Elements takes 7 or 11 positional fields, got %d" % len(vals))
            for f, q in zip(self.ALL_FIELDS, vals):
                setattr(self, f, q)
            return
        kw = {self._ALIASES.get(k, k): v for k, v in kw.items()}
        unknown = set(kw) - set(self.ALL_FIELDS)
        if unknown:
            raise TypeError("unknown Elements keyword(s): %s" % ", ".join(sorted(unknown)))
        if "m" not in kw:
            raise TypeError("Elements needs the keyword m")
        self._from_keywords(**kw)

    def _from_keywords(self, m, P=math.nan, t0=math.nan, ecosw=math.nan, esinw=math.nan, I=math.nan,
                       Omega=math.nan, a=math.nan, w=math.nan, e=math.nan, tp=math.nan):
        """The keyword constructor (InitialConditions.jl:64-107)."""
        m, P, t0, ecosw, esinw, I, Omega, a, w, e, tp = (float(q) for q in (m, P, t0, ecosw, esinw, I, Omega, a, w,
                                                                              e, tp))
        vals = [P, t0, ecosw, esinw, I, Omega, a, w, e, tp]
        if all(math.isnan(q) for q in vals):
            self.m, self.P, self.t0, self.ecosw, self.esinw, self.I, self.Omega = m, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0
            self.a = self.e = self.w = self.tp = 0.0
            return
        if math.isnan(P) and math.isnan(a):
            raise ValueError("Must specify either P or a.")
        if P > 0 and a > 0:
            raise ValueError("Only one of P (period) or a (semi-major axis) can be defined")
        if P < 0:
            raise ValueError("Period must be positive")
        if a < 0:
            raise ValueError("Orbital semi-major axis must be positive")
        if not math.isnan(e) and not (0.0 <= e < 1.0):
            raise ValueError("Eccentricity must be in [0,1), e=%r" % e)
        if not (math.isnan(ecosw) and math.isnan(esinw)) and not math.isnan(e):
            raise ValueError("Must specify either e and ecosw/esinw, but not both.")
        if not (math.isnan(tp) or math.isnan(t0)):
            raise ValueError("Must specify either initial transit time or time of periastron passage, but not both.")
        w = 0.0 if math.isnan(w) else w
        if math.isnan(e) and math.isnan(ecosw) and math.isnan(esinw):
            e = ecosw = esinw = 0.0
        if math.isnan(e):
            ecosw = 0.0 if math.isnan(ecosw) else ecosw
            esinw = 0.0 if math.isnan(esinw) else esinw
            e = math.sqrt(ecosw * ecosw + esinw * esinw)
            if not (0.0 <= e < 1.0):
                raise ValueError("Eccentricity must be in [0,1)")
            w = math.atan2(esinw, ecosw)
        else:
            esinw, ecosw = e * math.sin(w), e * math.cos(w)
            eps = np.finfo(float).eps
            esinw = 0.0 if abs(esinw) < eps else esinw
            ecosw = 0.0 if abs(ecosw) < eps else ecosw
        t0 = 0.0 if math.isnan(t0) else t0
        n = _ieee_div(2 * math.pi, P)
        if math.isnan(tp) and e != 0:
            tp = _ieee_rem(t0 - _ieee_div(math.sqrt(1.0 - e * e) * ecosw, n * (1.0 - esinw)) -
                           _ieee_div(2.0, n) * math.atan2(math.sqrt(1.0 - e) * (esinw + ecosw + e),
                                                          math.sqrt(1.0 + e) * (esinw - ecosw - e)), P)
        elif math.isnan(tp):
            tp = _ieee_div(math.pi / 2 + w, n)
        self.m, self.P, self.t0, self.ecosw, self.esinw = m, P, t0, ecosw, esinw
        self.I = 0.0 if math.isnan(I) else I
        self.Omega = 0.0 if math.isnan(Omega) else Omega
        self.a = 0.0 if math.isnan(a) else a
        self.e, self.w, self.tp = e, w, tp

    def row(self):
        return [self.m, self.P, self.t0, self.ecosw, self.esinw, self.I, self.Omega]


def hierarchy_nested(N):
    """Fully nested hierarchy matrix (what hierarchy([N, 1, ..., 1]) returns)."""
    H = np.zeros((N, N))
    for i in range(N - 1):
        H[i, :i + 1] = -1.0
        H[i, i + 1] = 1.0
    H[N - 1, :] = -1.0
    return H


class _Rows:
    """Writes 1-based rows and inclusive column ranges of an N x N matrix, as the hierarchy builder's indexing
    reads; an index outside the matrix is an invalid hierarchy (the reference stops with a BoundsError)."""

    def __init__(self, n):
        self.n = n
        self.h = np.zeros((n, n))

    def _check(self, r, c):
        if not (1 <= r <= self.n and 1 <= c <= self.n):
            raise ValueError("Invalid hierarchy: entry (%d, %d) outside the %d x %d matrix" % (r, c, self.n, self.n))

    def put(self, r, c, val):
        self._check(r, c)
        self.h[r - 1, c - 1] = val

    def fill(self, r, c1, c2, val):
        """Columns c1..c2 of row r (none when c2 < c1)."""
        if c2 < c1:
            return
        self._check(r, c1)
        self._check(r, c2)
        self.h[r - 1, c1 - 1:c2] = val


def _whole(x):
    """An integer-valued quotient (the reference converts it to Int64, which fails for a fraction)."""
    if x != int(x):
        raise ValueError("Invalid hierarchy: %g bodies do not split evenly" % x)
    return int(x)


def hierarchy(ic_vec):
    """Hierarchy matrix from a hierarchy vector [N, b1, b2, ...], b_k binaries on level k (setup_hierarchy.jl:9-179).

    The same level-filling rules and limits as the reference: the first level pairs bodies left to right, a
    hierarchy with every body on the bottom level (2 b1 = N) or with more than one binary on its top level is
    filled symmetrically, and any other fills one level after another, with at most two binaries on a level.
    [N, 1, ..., 1] gives the fully nested matrix, [4, 2, 1] two binaries orbiting each other.
    """
    v = [int(q) for q in ic_vec]
    if len(v) < 2:
        raise ValueError("Invalid hierarchy: [N, binaries on level 1, ...] needs at least two entries")
    nbody, bins = v[0], v[1:]
    level = len(bins) if bins[-1] == 1 else len(bins) - 1
    if not (bins[0] <= nbody / 2 and bins[0] <= 2 ** level):
        raise ValueError("Invalid hierarchy.")
    if sum(bins[:level]) != nbody - 1:
        raise ValueError("Invalid hierarchy. Total # of binaries should = N-1")
    w = _Rows(nbody)
    # first level (setup_hierarchy.jl:34-62): binaries (1,2), (3,4), ... left to right
    w.put(1, 1, -1.0)
    w.put(1, 2, 1.0)
    if bins[0] > 1:
        j = 1 if bins[-1] == 1 else _whole(nbody / 2 - 1)
        for i in range(1, bins[0]):
            if j + 3 <= nbody:
                w.put(i + 1, j + 2, -1.0)
                w.put(i + 1, j + 3, 1.0)
                j += 2
    binsp, row, bodies = bins[0], bins[0] + 1, 2 * bins[0]
    if bins[-1] > 1:
        _hierarchy_symmetric_nest(w, nbody, row)
    elif 2 * binsp == nbody:
        _hierarchy_symmetric(w, nbody, binsp, row)
    else:
        _hierarchy_levels(w, nbody, bodies, bins, binsp, row)
    w.h[nbody - 1, :] = -1.0
    return w.h


def _hierarchy_levels(w, nbody, bodies, bins, binsp, row):
    """Levels 2, 3, ... one after another (nlevel, setup_hierarchy.jl:71-145): `bodies` counts the bodies
    placed so far, `binsp` the binaries of the previous level; filling stops where the rules have no case."""
    it = 2
    while it <= len(bins):
        b = bins[it - 1]
        if nbody != bodies:
            if b == binsp:
                bodies += b
            elif b > binsp:
                bodies += 2 * b - 1
        elif row == nbody - 1:  # every body placed: the last row below the top joins the two halves
            if bodies % 4 > 2:
                w.fill(row, 1, row - 2, -1.0)
                w.fill(row, row - 1, bodies, 1.0)
            else:
                w.fill(row, 1, row - 1, -1.0)
                w.fill(row, row, bodies, 1.0)
            return
        if nbody < bodies:
            return
        if binsp == 1 and b == 1:
            w.fill(row, 1, bodies - binsp, -1.0)
            w.fill(row, bodies - binsp + 1, bodies, 1.0)
            row += binsp
        elif binsp == 1 and b == 2:
            w.fill(row, 1, bodies - 2 * binsp - 1, -1.0)
            w.put(row, bodies - 2 * binsp, 1.0)
            w.put(row + 1, bodies - 2 * binsp + 1, -1.0)
            w.put(row + 1, bodies, 1.0)
            row += 2
        elif binsp == 2 and b == 1:
            w.fill(row, 1, row - 1, -1.0)
            w.fill(row, row, bodies, 1.0)
            row += 1
        elif binsp == 2 and b == 2:
            w.fill(row, 1, row - 1, -1.0)
            w.fill(row, row, bodies - 2 * (binsp - 1), 1.0)
            w.put(row + 1, bodies - 2 * (binsp - 1) + 1, -1.0)
            w.put(row + 1, bodies, 1.0)
            row += 2
        elif binsp == 3 and b == 2:
            half, third = _whole(bodies / 2), _whole(bodies / 3)
            w.fill(row, 1, half - 1, -1.0)
            w.fill(row, half, 2 * third, 1.0)
            w.fill(row + 1, 2 * third + 1, bodies, -1.0)
            w.put(row + 1, bodies + 1, 1.0)
            row += 2
            bodies += 1
        else:
            return
        binsp = b
        it += 1


def _hierarchy_symmetric(w, nbody, binsp, row):
    """Every body on the bottom level (symmetric, setup_hierarchy.jl:151-164): pairs of binaries join four
    bodies at a time, then the top row splits the system after its first binsp bodies."""
    j = 0
    while row < nbody - 1:
        w.fill(row, 1 + j, 2 + j, -1.0)
        w.fill(row, j + 3, j + 4, 1.0)
        j += 4
        row += 1
    w.fill(row, 1, binsp, -1.0)
    w.fill(row, binsp + 1, nbody, 1.0)


def _hierarchy_symmetric_nest(w, nbody, row):
    """More than one binary on the top level (symmetric_nest, setup_hierarchy.jl:166-179): both halves grow
    a nested sequence side by side, then the top row joins the halves."""
    hlf = _whole(nbody / 2)
    j = 0
    while row < nbody - 1:
        w.fill(row, 1, 2 + j, -1.0)
        w.put(row, 3 + j, 1.0)
        w.fill(row + 1, hlf + 1, hlf + 2 + j, -1.0)
        w.put(row + 1, hlf + 3 + j, 1.0)
        j += 1
        row += 2
    w.fill(row, 1, hlf, -1.0)
    w.fill(row, hlf + 1, nbody, 1.0)


def _sigma_m(m, i, j, H):
    s = 0.0
    for l in range(len(m)):
        s = s + m[l] * (1.0 if H[i, j] == H[i, l] else 0.0)
    return s


def amatrix(H, m):
    """A matrix of Hamers & Portegies Zwart 2016 (init_nbody.jl:176-184)."""
    N = len(m)
    A = np.zeros((N, N))
    for i in range(N):
        for j in range(N):
            A[i, j] = (H[i, j] * m[j]) / _sigma_m(m, i, j, H)
    return A


def _jmod(x, y):
    r = math.fmod(x, y)
    if r == 0.0:
        return math.copysign(0.0, y)
    if (r > 0) != (y > 0):
        return r + y
    return r


def ekepler(m, ecc):
    """Eccentric anomaly from mean anomaly (kepler.jl:1-41)."""
    if m == 0.0:
        return 0.0
    ms = _jmod(m, 2 * math.pi)
    sg = 1.0 if ms > 0 else (-1.0 if ms < 0 else 0.0)
    de0 = ecc * 0.85 * sg
    de1, de2 = 2 * de0, 3 * de0
    it = 0
    while True:
        de2 = de1
        de1 = de0
        f3 = ecc * math.cos(de0 + ms)
        f2 = ecc * math.sin(de0 + ms)
        de0 = (f2 - de1 * f3) / (1.0 - f3)
        it += 1
        if it >= 20 or de0 == de1 or de0 == de2:
            break
    return de0 + m


def kepler_init(time, mass, el):
    """Position, velocity and 7x7 Jacobian of one Keplerian (kepler_init.jl:66-210)."""
    period, t0, ecosw, esinw, inc, capom = (float(q) for q in el)
    n = 2 * math.pi / period
    semi = math.cbrt(GNEWT * mass * (period * period) / 4 / (math.pi * math.pi))
    dsemidp = 2 * THIRD * semi / period
    dsemidm = THIRD * semi / mass
    ecc = math.sqrt(esinw * esinw + ecosw * ecosw)
    deccdecos = ecosw / ecc if ecc != 0 else 0.0
    deccdesin = esinw / ecc if ecc != 0 else 0.0
    sq = math.sqrt(1.0 - ecc * ecc)
    den1 = esinw - ecosw - ecc
    if ecc == 0.0:
        tp = t0 - 3 * period / 4
    else:
        tp = (t0 - sq / n * ecosw / (1.0 - esinw) -
              2 / n * math.atan2(math.sqrt(1.0 - ecc) * (esinw + ecosw + ecc), math.sqrt(1.0 + ecc) * den1))
    dtpdp = (tp - t0) / period
    fac = math.sqrt((1.0 - ecc) / (1.0 + ecc))
    den2 = 1.0 / (den1 * den1) if den1 != 0 else math.inf
    theta = fac * (esinw + ecosw + ecc) / den1 if den1 != 0 else math.inf
    with np.errstate(all="ignore"):
        dthetadecc = (((ecc + ecosw) ** 2 + 2 * (1.0 - ecc * ecc) * esinw - esinw * esinw) /
                      (sq * (1.0 + ecc)) * den2)
        dthetadecos = 2 * fac * esinw * den2
        dthetadesin = -(2 * fac) * (ecosw + ecc) * den2
        th2 = 1.0 + theta * theta
        dtpdecc = ecc / sq / n * ecosw / (1.0 - esinw) - 2 / n / th2 * dthetadecc
        dtpdecos = dtpdecc * deccdecos - sq / n / (1.0 - esinw) - 2 / n / th2 * dthetadecos
        dtpdesin = (dtpdecc * deccdesin - sq / n * ecosw / ((1.0 - esinw) * (1.0 - esinw)) -
                    2 / n / th2 * dthetadesin)
    m = n * (time - tp)
    dmdp = -m / period
    dmdtp = -n
    ekep = ekepler(m, ecc)
    ce, se = math.cos(ekep), math.sin(ekep)
    r = semi * (1.0 - ecc * ce)
    denom = semi / r
    dekepdecos = se * denom * deccdecos
    dekepdesin = se * denom * deccdesin
    dekepdm = denom
    cO, sO = math.cos(capom), math.sin(capom)
    cw = ecosw / ecc if ecc != 0 else 1.0
    sw = esinw / ecc if ecc != 0 else 0.0
    ci, si = math.cos(inc), math.sin(inc)
    P1 = np.array([[cw, -sw, 0.0], [sw, cw, 0.0], [0.0, 0.0, 1.0]])
    P2 = np.array([[1.0, 0.0, 0.0], [0.0, ci, -si], [0.0, si, ci]])
    P3 = np.array([[cO, -sO, 0.0], [sO, cO, 0.0], [0.0, 0.0, 1.0]])
    P32 = P3 @ P2
    P321 = P32 @ P1
    xplane = np.array([semi * (ce - ecc), semi * (sq * se), 0.0])
    vplane = np.array([-se, sq * ce, 0.0])
    x = P321 @ xplane
    nsd = n * semi * denom
    v = (P321 * nsd) @ vplane
    J = np.zeros((7, 7))
    dxda = x / semi
    dxdekep = (P321 * semi) @ vplane
    Dinc = np.array([[0.0, 0.0, 0.0], [0.0, -si, -ci], [0.0, ci, -si]])
    Dcom = np.array([[-sO, -cO, 0.0], [cO, -sO, 0.0], [0.0, 0.0, 0.0]])
    dxdinc = (P3 @ Dinc @ P1) @ xplane
    dxdcom = (Dcom @ P2 @ P1) @ xplane
    dvda = v / semi
    dvdp = -v / period
    dvdekep = -v * ecc * se * denom + (P321 * nsd) @ np.array([-ce, -sq * se, 0.0])
    dvdinc = ((P3 @ Dinc @ P1) * nsd) @ vplane
    dvdcom = ((Dcom @ P2 @ P1) * nsd) @ vplane
    J[0:3, 0] = dxda * dsemidp + dxdekep * dekepdm * (dmdp + dmdtp * dtpdp)
    J[0:3, 1] = dxdekep * dekepdm * dmdtp * 1.0
    J[3:6, 0] = dvdp + dvda * dsemidp + dvdekep * dekepdm * (dmdp + dmdtp * dtpdp)
    J[3:6, 1] = dvdekep * dekepdm * dmdtp * 1.0
    if ecc != 0.0:
        dxdecc = ((-P321) * semi / ecc) @ np.array([ce, se / sq, 0.0])
        dxdecos = dxdecc * deccdecos + (P32 / ecc) @ xplane
        dxdesin = dxdecc * deccdesin + (P32 / ecc) @ np.array([-xplane[1], xplane[0], 0.0])
        dvdecc = -v / ecc + v * ce * denom + (P321 * nsd) @ np.array([0.0, -ecc / sq * ce, 0.0])
        dvdecos = dvdecc * deccdecos + ((P32 * nsd) / ecc) @ vplane
        dvdesin = dvdecc * deccdesin + ((P32 * nsd) / ecc) @ np.array([-vplane[1], vplane[0], 0.0])
        J[0:3, 2] = dxdecos + dxdekep * (dekepdm * dmdtp * dtpdecos + dekepdecos)
        J[0:3, 3] = dxdesin + dxdekep * (dekepdm * dmdtp * dtpdesin + dekepdesin)
        J[3:6, 2] = dvdecos + dvdekep * (dekepdm * dmdtp * dtpdecos + dekepdecos)
        J[3:6, 3] = dvdesin + dvdekep * (dekepdm * dmdtp * dtpdesin + dekepdesin)
    J[0:3, 4] = dxdinc
    J[0:3, 5] = dxdcom
    J[0:3, 6] = dxda * dsemidm
    J[3:6, 4] = dvdinc
    J[3:6, 5] = dvdcom
    J[3:6, 6] = dvda * dsemidm
    J[6, 6] = 1.0
    return x, v, J


def init_nbody(elements, t0, H):
    """x (3xN), v (3xN), jac_init (7Nx7N) for an ElementsIC (init_nbody.jl:13-162)."""
    el = np.asarray(elements, dtype=np.float64)
    N = H.shape[0]
    M = 7 * N
    m = el[:N, 0].copy()
    A = amatrix(H, m)
    Ainv = np.linalg.inv(A)
    rk = np.zeros((N, 3))
    rdk = np.zeros((N, 3))
    jk = np.zeros((6 * N, M))
    i, b = 0, 0
    while i < N - 1:
        ind = H[i, :] != 0
        mu = 0.0
        for l in range(N):
            if ind[l]:
                mu = mu + m[l]
        if H[i, 0] == 0:
            b += 1
        r, rd, j21 = kepler_init(t0, mu, el[i + 1 + b, 1:7])
        rk[i, :] = r
        rdk[i, :] = rd
        jk[6 * i:6 * i + 6, 7 * (i + 1):7 * (i + 1) + 6] = j21[0:6, 0:6]
        for j in range(N):
            if H[i, j] != 0:
                jk[6 * i:6 * i + 6, 7 * j + 6] = j21[0:6, 6]
        if b > 0:
            b -= 2
        elif b < 0:
            b = 0
        i += 1
    jac = np.zeros((M, M))
    dAdm = np.zeros((N, N, N))
    for k in range(N):
        for ii in range(N):
            for j in range(N):
                sm = _sigma_m(m, ii, j, H)
                dkj = 1.0 if k == j else 0.0
                dee = 1.0 if H[ii, j] == H[ii, k] else 0.0
                dAdm[ii, j, k] = (dkj * H[ii, j]) / sm - dee * H[ii, j] * m[j] / (sm * sm)
    dAinvdm = np.zeros((N, N, N))
    for k in range(N):
        dAinvdm[:, :, k] = (-Ainv) @ dAdm[:, :, k] @ Ainv
    for ii in range(N):
        for k in range(N):
            jac[7 * ii:7 * ii + 3, :] += Ainv[ii, k] * jk[6 * k:6 * k + 3, :]
            jac[7 * ii + 3:7 * ii + 6, :] += Ainv[ii, k] * jk[6 * k + 3:6 * k + 6, :]
        for k in range(N):
            dxdm = dAinvdm[:, :, k] @ rk
            dvdm = dAinvdm[:, :, k] @ rdk
            jac[7 * ii:7 * ii + 3, 7 * k + 6] += dxdm[ii, :]
            jac[7 * ii + 3:7 * ii + 6, 7 * k + 6] += dvdm[ii, :]
        jac[7 * ii + 6, 7 * ii + 6] = 1.0
    x = np.asfortranarray((Ainv @ rk).T)
    v = np.asfortranarray((Ainv @ rdk).T)
    return x, v, np.asfortranarray(jac)


def _read_rows(path, comments):
    """A comma-separated numeric file as a matrix (readdlm(path, ',') with or without '#' comment lines)."""
    return np.loadtxt(path, delimiter=",", comments="#" if comments else None, ndmin=2)


class ElementsIC:
    """Initial conditions from a hierarchy and orbital elements (InitialConditions.jl:142-241).

    H may be an int N (fully nested), a hierarchy vector [N, b1, b2, ...]
    (hierarchy()), or a hierarchy matrix.  elements is an N x 7 array (more
    rows are allowed; the first N are used), a list of Elements (one per body,
    in hierarchy order, missing bodies zero), or the name of a comma-separated
    file with '#' comment lines.
    """

    def __init__(self, t0, H, *elements, der=True):
        if isinstance(H, (int, np.integer)):
            Hm = hierarchy_nested(int(H))
        else:
            Ha = np.asarray(H)
            if Ha.ndim == 1:
                Hm = hierarchy([int(q) for q in Ha])
            elif Ha.ndim == 2:
                Hm = np.array(Ha, dtype=np.float64)
            else:
                raise ValueError("H must be a body count, a hierarchy vector or a hierarchy matrix")
        nbody = Hm.shape[0]
        if len(elements) == 1 and isinstance(elements[0], (str, os.PathLike)):
            el = _read_rows(elements[0], comments=True)
        elif len(elements) == 1 and not isinstance(elements[0], (Elements, list, tuple)):
            el = np.array(elements[0], dtype=np.float64)
        else:
            els = elements[0] if (len(elements) == 1 and isinstance(elements[0], (list, tuple))) else elements
            el = np.zeros((nbody, 7))
            for i, e in enumerate(els):  # InitialConditions.jl:213-220: unlisted bodies stay zero
                el[i] = e.row()
        self.elements = np.array(el[:nbody, :], dtype=np.float64)
        self.H = Hm
        self.nbody = nbody
        self.m = self.elements[:, 0].copy()
        self.amat = amatrix(Hm, self.m)
        self.t0 = float(t0)
        self.der = der

    def init_nbody(self):
        return init_nbody(self.elements, self.t0, self.H)


class CartesianIC:
    """Initial conditions from Cartesian coordinates (InitialConditions.jl:259-282): rows (m, x, y, z, vx, vy,
    vz), as a matrix or the name of a comma-separated file (read without comment lines, as the reference)."""

    def __init__(self, t0, N, coords):
        if isinstance(coords, (str, os.PathLike)):
            c = _read_rows(coords, comments=False)
        else:
            c = np.array(coords, dtype=np.float64)
        self.m = c[:N, 0].copy()
        self.x = np.asfortranarray(c[:N, 1:4].T)
        self.v = np.asfortranarray(c[:N, 4:7].T)
        self.nbody = N
        self.t0 = float(t0)

    def init_nbody(self):
        return self.x.copy(order="F"), self.v.copy(order="F"), np.asfortranarray(np.eye(7 * self.nbody))
