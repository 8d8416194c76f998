"""Independent transliteration of the reference in high precision (test infrastructure only).

A second restatement of BlackSiberian/HyperelasticSolver's hot path, written
function by function after the Julia source and evaluated in mpmath at 40
significant digits with its own forward-mode dual numbers (the algorithm of
ForwardDiff.jl). It shares no code with ``hyp_oracle.hpp``; the tests use it to
check that the C++ oracle computes the reference's mathematics (agreement to
rounding level), and ``tests/golden/make_golden.py`` uses it to write the
committed golden vectors. Pure-Python loops: small cases only.

Citations are to files of the reference project.
"""
import mpmath as mp

mp.mp.dps = 40


class D:
    """Forward-mode dual number: value ``v`` and partials list ``d``.

    Values and partials may themselves be ``D`` (nesting = ForwardDiff's
    jacobian-of-gradient in EquationsOfState.jl:200,226)."""

    __slots__ = ("v", "d")

    def __init__(self, v, d):
        self.v, self.d = v, d

    @staticmethod
    def lift(x, n):
        return x if isinstance(x, D) else D(x, [0] * n)

    def _n(self):
        return len(self.d)

    def __add__(a, b):
        if not isinstance(b, D):
            return D(a.v + b, a.d)
        return D(a.v + b.v, [x + y for x, y in zip(a.d, b.d)])

    __radd__ = __add__

    def __neg__(a):
        return D(-a.v, [-x for x in a.d])

    def __sub__(a, b):
        return a + (-b)

    def __rsub__(a, b):
        return (-a) + b

    def __mul__(a, b):
        if not isinstance(b, D):
            return D(a.v * b, [x * b for x in a.d])
        return D(a.v * b.v, [x * b.v + y * a.v for x, y in zip(a.d, b.d)])

    __rmul__ = __mul__

    def __truediv__(a, b):
        if not isinstance(b, D):
            return D(a.v / b, [x / b for x in a.d])
        return D(a.v / b.v, [x / b.v - y * (a.v / (b.v * b.v)) for x, y in zip(a.d, b.d)])

    def __rtruediv__(a, b):  # b / a with b a constant
        return D(b / a.v, [-(b / (a.v * a.v)) * x for x in a.d])

    def __pow__(a, p):  # real exponent
        return D(a.v ** p, [x * p * a.v ** (p - 1) for x in a.d])

    def __lt__(a, b):
        return val(a) < val(b)

    def __gt__(a, b):
        return val(a) > val(b)


def val(x):
    while isinstance(x, D):
        x = x.v
    return x


def dsqrt(x):
    if isinstance(x, D):
        s = dsqrt(x.v)
        return D(s, [y / (2 * s) for y in x.d])
    return mp.sqrt(x)


def dexp(x):
    if isinstance(x, D):
        e = dexp(x.v)
        return D(e, [e * y for y in x.d])
    return mp.exp(x)


def dlog(x):
    if isinstance(x, D):
        return D(dlog(x.v), [y / x.v for y in x.d])
    return mp.log(x)


def dabs(x):
    return -x if val(x) < 0 else x


def seed(xs):
    n = len(xs)
    return [D(x, [1 if j == i else 0 for j in range(n)]) for i, x in enumerate(xs)]


# --- SimpleLA.jl / Strains.jl (column-major 9-vectors, m(i,j) = m[i + 3j]) ---
def mget(m, i, j):
    return m[i + 3 * j]


def det_(m):  # SimpleLA.jl:84-89
    g = lambda i, j: mget(m, i, j)  # noqa: E731
    return (g(0, 0) * (g(1, 1) * g(2, 2) - g(2, 1) * g(1, 2)) - g(0, 1) * (g(1, 0) * g(2, 2) - g(1, 2) * g(2, 0))
            + g(0, 2) * (g(1, 0) * g(2, 1) - g(1, 1) * g(2, 0)))


def inv_(m):  # SimpleLA.jl:51-79
    g = lambda i, j: mget(m, i, j)  # noqa: E731
    invdet = 1 / det_(m)
    r = [None] * 9
    r[0 + 0] = (g(1, 1) * g(2, 2) - g(2, 1) * g(1, 2)) * invdet
    r[0 + 3] = (g(0, 2) * g(2, 1) - g(0, 1) * g(2, 2)) * invdet
    r[0 + 6] = (g(0, 1) * g(1, 2) - g(0, 2) * g(1, 1)) * invdet
    r[1 + 0] = (g(1, 2) * g(2, 0) - g(1, 0) * g(2, 2)) * invdet
    r[1 + 3] = (g(0, 0) * g(2, 2) - g(0, 2) * g(2, 0)) * invdet
    r[1 + 6] = (g(1, 0) * g(0, 2) - g(0, 0) * g(1, 2)) * invdet
    r[2 + 0] = (g(1, 0) * g(2, 1) - g(2, 0) * g(1, 1)) * invdet
    r[2 + 3] = (g(2, 0) * g(0, 1) - g(0, 0) * g(2, 1)) * invdet
    r[2 + 6] = (g(0, 0) * g(1, 1) - g(1, 0) * g(0, 1)) * invdet
    return r


def _mm(a, b, i, j):
    return mget(a, i, 0) * mget(b, 0, j) + mget(a, i, 1) * mget(b, 1, j) + mget(a, i, 2) * mget(b, 2, j)


def tr_(m):
    return mget(m, 0, 0) + mget(m, 1, 1) + mget(m, 2, 2)


def det_lu(m):
    """LinearAlgebra.det (LU, partial pivoting)."""
    a = [[mget(m, i, j) for j in range(3)] for i in range(3)]
    sign = 1
    for k in range(3):
        kp = max(range(k, 3), key=lambda i: abs(val(a[i][k])))
        if val(a[kp][k]) == 0:
            return 0 * a[0][0]
        if kp != k:
            a[k], a[kp] = a[kp], a[k]
            sign = -sign
        for i in range(k + 1, 3):
            a[i][k] = a[i][k] / a[k][k]
            for j in range(k + 1, 3):
                a[i][j] = a[i][j] - a[i][k] * a[k][j]
    return a[0][0] * a[1][1] * a[2][2] * sign


def finger(a):  # Strains.jl:26-32
    at = [None] * 9
    for i in range(3):
        for j in range(3):
            at[i + 3 * j] = mget(a, j, i)
    return inv_([_mm(a, at, i, j) for j in range(3) for i in range(3)])


def invariants(g):  # Strains.jl:46-52
    g2 = [_mm(g, g, i, j) for j in range(3) for i in range(3)]
    return [tr_(g), (tr_(g) * tr_(g) - tr_(g2)) / 2, det_(g)]


# --- EquationsOfState.jl ---
class Barton:
    def __init__(self, rho0=8.93, c0=4.6, cv=3.9e-4, t0=300, b0=2.1, alpha=1, beta=3, gamma=2):
        mpf = mp.mpf
        self.rho0, self.c0, self.cv, self.t0, self.b0 = mpf(rho0), mpf(c0), mpf(cv), mpf(t0), mpf(b0)
        self.alpha, self.beta, self.gamma = mpf(alpha), mpf(beta), mpf(gamma)
        self.b0sq = self.b0 ** 2
        self.k0 = self.c0 ** 2 - mpf(4) / 3 * self.b0 ** 2


def energy(e, S, G):  # :118-137
    i1, i2, i3 = invariants(G)
    U = e.k0 / (2 * e.alpha ** 2) * (i3 ** (e.alpha / 2) - 1) * (i3 ** (e.alpha / 2) - 1) + \
        e.cv * e.t0 * i3 ** (e.gamma / 2) * (dexp(S / e.cv) - 1)
    W = e.b0sq / 2 * i3 ** (e.beta / 2) * (i1 * i1 / 3 - i2)
    return U + W


def entropy(e, eint, G):  # :139-156
    i1, i2, i3 = invariants(G)
    S = eint - e.b0sq / 2 * i3 ** (e.beta / 2) * (i1 * i1 / 3 - i2) - \
        e.k0 / (2 * e.alpha ** 2) * (i3 ** (e.alpha / 2) - 1) * (i3 ** (e.alpha / 2) - 1)
    S = S / (e.cv * e.t0 * i3 ** (e.gamma / 2)) + 1
    if val(S) < mp.mpf("1e-6"):
        S = mp.mpf("1e-6")
    return dlog(S) * e.cv


def gradient(f, x):
    r = f(seed(x))
    return list(r.d)


def stress(e, ent, F):  # :179-190
    den = e.rho0 / det_lu(F)
    G = finger(F)
    dedG = gradient(lambda g: energy(e, ent, g), G)
    a = [-2 * den * g for g in G]
    return [_mm(a, dedG, i, j) for j in range(3) for i in range(3)]


def acoustic(e, ent, F, n=(1, 0, 0)):  # :223-246
    sd = stress(e, ent, seed(F))
    den = e.rho0 / det_lu(F)
    ac = [None] * 9
    for i in range(3):
        for j in range(3):
            ac[i + 3 * j] = sum(sd[m + 3 * i].d[j + 3 * l] / den * mget(F, k, l) * n[m] * n[k]
                                for k in range(3) for l in range(3) for m in range(3) if n[m] != 0 and n[k] != 0)
    return ac


def stress_den(e, den, eint, F):  # :162-176, the entropy from e_int, den given
    G = finger(F)
    S = entropy(e, eint, G)
    dedG = gradient(lambda g: energy(e, S, g), G)
    a = [-2 * den * g for g in G]
    return [_mm(a, dedG, i, j) for j in range(3) for i in range(3)]


def acoustic_prim(e, P, n):  # :192-221
    """acoustic(eos, P, n): the Jacobian of stress(eos, den, e_int, F) over F (den = P[1]
    P[2] and e_int = energy(eos, S, finger(F)) held), here by central differences in
    40-digit arithmetic (step 1e-15: truncation ~1e-30, cancellation ~1e-25), so this
    check shares neither the dual numbers nor the closed forms of the other restatements."""
    den = P[0] * P[1]
    F = list(P[6:15])
    eint = energy(e, P[5], finger(F))
    h = mp.mpf("1e-15")
    J = [[None] * 9 for _ in range(9)]  # J[p][q] = d sigma_p / d F_q
    for q in range(9):
        Fp, Fm = list(F), list(F)
        Fp[q] += h
        Fm[q] -= h
        sp, sm = stress_den(e, den, eint, Fp), stress_den(e, den, eint, Fm)
        for p_ in range(9):
            J[p_][q] = (sp[p_] - sm[p_]) / (2 * h)
    ac = [None] * 9
    for i in range(3):
        for j in range(3):
            ac[i + 3 * j] = sum(J[m + 3 * i][j + 3 * l] / den * mget(F, k, l) * n[m] * n[k]
                                for k in range(3) for l in range(3) for m in range(3))
    return ac


def eig_moduli(M):
    """Eigenvalue moduli of a real 3x3 (mpmath eig at 40 digits) in the order Julia's
    eigvals returns the eigenvalues (HyperelasticityMPh.jl:263): LinearAlgebra's default
    lexicographic sort by (real, imag)."""
    A = mp.matrix(3, 3)
    for i in range(3):
        for j in range(3):
            A[i, j] = val(mget(M, i, j))
    ev = mp.eig(A, left=False, right=False)
    ev = sorted(ev, key=lambda z: (mp.re(z), mp.im(z)))
    return [abs(x) for x in ev]


# --- HyperelasticityMPh.jl (one phase, 15-vector) ---
def cons2prim(e, Q):  # :106-133
    frac = Q[0]
    true_den = dsqrt(det_lu([q / frac for q in Q[6:15]]) / e.rho0)
    den = frac * true_den
    vel = [q / den for q in Q[2:5]]
    e_tot = Q[5] / den
    e_int = e_tot - (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]) / 2
    A = [q / den for q in Q[6:15]]
    return [frac, true_den] + vel + [entropy(e, e_int, finger(A))] + A


def prim2cons(e, P):  # :66-87
    frac, true_den = P[0], P[1]
    den = frac * true_den
    vel = P[2:5]
    eint = energy(e, P[5], finger(P[6:15]))
    etot = eint + (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]) / 2
    return [frac, den] + [den * v for v in vel] + [den * etot] + [den * a for a in P[6:15]]


def flux(e, Q):  # :146-175
    P = cons2prim(e, Q)
    frac, true_den, vel, ent, A = P[0], P[1], P[2:5], P[5], P[6:15]
    den = frac * true_den
    e_tot = Q[5] / den
    strs = [frac * s for s in stress(e, ent, A)]
    row = [strs[0], strs[3], strs[6]]
    out = [0, den * vel[0]]
    out += [den * vel[0] * vel[a] - row[a] for a in range(3)]
    out += [den * vel[0] * e_tot - sum(vel[a] * row[a] for a in range(3))]
    for b in range(3):
        for a in range(3):
            out.append(den * (vel[0] * mget(A, a, b) - vel[a] * mget(A, 0, b)))
    return out


def speeds(e, Q, n=(1, 0, 0)):  # :258-266
    P = cons2prim(e, Q)
    mods = eig_moduli(acoustic(e, P[5], P[6:15], n))
    c = [mp.sqrt(m) for m in mods]
    un = P[2] * n[0] + P[3] * n[1] + P[4] * n[2]
    return [un + x for x in c] + [un - x for x in c]


def noncons_cols(eos, Q):  # :178-250 (columns 1 and 16 of B)
    ph = [Q[0:15], Q[15:30]]
    P = [cons2prim(eos[p], ph[p]) for p in range(2)]
    frac = [P[p][0] for p in range(2)]
    td = [P[p][1] for p in range(2)]
    vel = [P[p][2:5] for p in range(2)]
    ent = [P[p][5] for p in range(2)]
    A = [P[p][6:15] for p in range(2)]
    G = [finger(A[p]) for p in range(2)]
    strs = [[frac[p] * s for s in stress(eos[p], ent[p], A[p])] for p in range(2)]
    temp = []
    for p in range(2):
        s = D(ent[p], [1])
        temp.append(energy(eos[p], s, [D(g, [0]) for g in G[p]]).d[0])
    k = [mp.mpf(1) / 2, 1 - mp.mpf(1) / 2]
    vel_i = [k[0] * vel[0][a] + k[1] * vel[1][a] for a in range(3)]
    K = [[s / frac[p] for s in strs[p]] for p in range(2)]
    si = [(k[1] * temp[1] * K[0][j] + k[0] * temp[0] * K[1][j]) / (k[0] * temp[0] + k[1] * temp[1]) for j in range(9)]
    out = []
    for p in range(2):
        b = [0] * 15
        b[0] = vel_i[0]
        for a in range(3):
            b[2 + a] = si[a]
        b[5] = sum(si[a] * vel_i[a] for a in range(3))
        for c in range(3):
            for a in range(3):
                b[6 + a + 3 * c] = td[p] * mget(A[p], 0, c) * vel[p][a]
        for c in range(3):
            b[6 + 3 * c] += td[p] * sum(mget(A[p], a, c) * (vel_i[a] - vel[p][a]) for a in range(3))
        out += b
    return out


def gauss_legendre6():
    x, w = zip(*[(mp.mpf(a), mp.mpf(b)) for a, b in _gl6()])
    return [(xi + 1) / 2 for xi in x], [wi / 2 for wi in w]


def _gl6():
    roots = sorted(mp.polyroots(mp.taylor(lambda t: mp.legendre(6, t), 0, 6)[::-1], maxsteps=200, extraprec=200))
    out = []
    for r in roots:
        r = mp.re(r)
        dp = mp.diff(lambda t: mp.legendre(6, t), r)
        out.append((r, 2 / ((1 - r * r) * dp * dp)))
    return out


def path_integral(eos, x, w, Qa, Qb):  # NumFluxes.jl:97-107
    dv = [b - a for a, b in zip(Qa, Qb)]
    acc = [0] * 30
    for s, wi in zip(x, w):
        u = [a * (1 - s) + b * s for a, b in zip(Qa, Qb)]
        bc = noncons_cols(eos, u)
        for r in range(30):
            acc[r] += wi * bc[r] * dv[0 if r < 15 else 15]
    return acc


def hll(eos, Ql, Qr, spdL, spdR):  # NumFluxes.jl:70-132
    Qm = [(a + b) / 2 for a, b in zip(Ql, Qr)]
    spdM = speeds(eos[0], Qm[:15]) + speeds(eos[1], Qm[15:])
    sl = min(0, min(spdM), min(spdL))
    sr = max(0, max(spdM), max(spdR))
    x, w = gauss_legendre6()
    fl = flux(eos[0], Ql[:15]) + flux(eos[1], Ql[15:])
    fr = flux(eos[0], Qr[:15]) + flux(eos[1], Qr[15:])
    b0 = path_integral(eos, x, w, Ql, Qr)
    pint = [b0[k] + fr[k] - fl[k] for k in range(30)]
    Qh = [(Qr[k] * sr - Ql[k] * sl - pint[k]) / (sr - sl) for k in range(30)]
    b1 = path_integral(eos, x, w, Ql, Qh)
    b2 = path_integral(eos, x, w, Qh, Qr)
    inner = [fr[k] - fl[k] + b1[k] + b2[k] for k in range(30)]
    dm = [-sl / (sr - sl) * inner[k] + sl * sr / (sr - sl) * (Qr[k] - Ql[k]) for k in range(30)]
    dp = [sr / (sr - sl) * inner[k] - sl * sr / (sr - sl) * (Qr[k] - Ql[k]) for k in range(30)]
    return dm, dp


def gauss_lobatto6():
    """Six-point Gauss-Lobatto rule on [0, 1] (FastGaussQuadrature's gausslobatto(6),
    NumFluxes.jl:36-37): the end points and the roots of P5', weights
    2 / (n (n - 1) P5(x)^2) on [-1, 1]."""
    d5 = lambda t: mp.diff(lambda y: mp.legendre(5, y), t)  # noqa: E731
    inner = sorted(mp.re(r) for r in mp.polyroots(mp.taylor(d5, 0, 4)[::-1], maxsteps=200, extraprec=200))
    x = [mp.mpf(-1)] + inner + [mp.mpf(1)]
    w = [mp.mpf(2) / (30 * mp.legendre(5, t) ** 2) for t in x]
    return [(xi + 1) / 2 for xi in x], [wi / 2 for wi in w]


def lxf2(eos, Ql, Qr, lam):  # NumFluxes.jl:25-60, two phases
    fl = flux(eos[0], Ql[:15]) + flux(eos[1], Ql[15:])
    fr = flux(eos[0], Qr[:15]) + flux(eos[1], Qr[15:])
    cons = [mp.mpf("0.5") * (fl[k] + fr[k]) - mp.mpf("0.5") * lam * (Qr[k] - Ql[k]) for k in range(30)]
    x, w = gauss_lobatto6()
    fp = path_integral(eos, x, w, Ql, Qr)
    half = [fp[k] / 2 for k in range(30)]
    return cons, half, list(half)


# --- Hank2016 (EquationsOfState.jl:305-366) ---
class Hank:
    def __init__(self, rho0=2.7, mu=26e9, gamma=3.4, pres_inf=21.5e9, a=0.5):
        self.rho0, self.mu, self.gamma = mp.mpf(rho0), mp.mpf(mu), mp.mpf(gamma)
        self.pres_inf, self.a = mp.mpf(pres_inf), mp.mpf(a)


def _hank_e_el(h, i):
    j1 = i[0] / i[2] ** (mp.mpf(1) / 3)
    j2 = (i[0] ** 2 - 2 * i[1]) / i[2] ** (mp.mpf(2) / 3)
    return h.mu / (4 * h.rho0) * ((1 - 2 * h.a) / 3 * j1 ** 2 + h.a * j2 + 3 * (h.a - 1))


def hank_energy(h, den, pres, G):  # :321-336
    return _hank_e_el(h, invariants(G)) + (pres + h.gamma * h.pres_inf) / (den * (h.gamma - 1))


def hank_pressure(h, den, e_int, i):  # :338-352
    return (e_int - _hank_e_el(h, i)) * (h.gamma - 1) * den - h.gamma * h.pres_inf


def hank_stress(h, den, pres, F):  # :354-361
    G = finger(inv_(F))
    dedG = gradient(lambda g: hank_energy(h, den, pres, g), G)
    a = [-2 * den * g for g in G]
    return [_mm(a, dedG, i, j) for j in range(3) for i in range(3)]


# --- single-phase (alpha == 1) Rusanov step of main.jl:202-227 on a small grid ---
def rusanov_step(e, Q, cfl, X=1, frozen=True):
    """Q: list of 14-vectors. Returns (new Q, dt)."""
    nx = len(Q)
    q15 = [[mp.mpf(1)] + list(q) for q in Q]
    lam = [max(abs(s) for s in speeds(e, q)) for q in q15]
    dx = mp.mpf(X) / nx
    dt = cfl * dx / max(lam)
    f = [flux(e, q)[1:] for q in q15]

    def F(i, j):  # face between cells i and j
        lf = max(lam[i], lam[j])
        return [(f[i][k] + f[j][k]) / 2 - lf / 2 * (Q[j][k] - Q[i][k]) for k in range(14)]

    out = [list(q) for q in Q]
    rng = range(1, nx - 1) if frozen else range(nx)
    for i in rng:
        il, ir = max(i - 1, 0), min(i + 1, nx - 1)
        Fl, Fr = F(il, i), F(i, ir)
        out[i] = [Q[i][k] - dt / dx * (Fr[k] - Fl[k]) for k in range(14)]
    return out, dt
