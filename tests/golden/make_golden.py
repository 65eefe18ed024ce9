"""Generates tests/golden/golden.json from independent pure-Python statements (no
oracle code): the reference's pair potentials (src/system/lj.rs:78-81, wca.rs:61-76)
with Rust's powi expansion, the specified Philox4x32-10 draw stream, the exact density of
states of a 4x4 periodic Ising lattice by enumeration (energy of ising.rs:59-75), and
heat capacities by plotting/final_heat_capacity.py:79-88 written in numpy.

    python tests/golden/make_golden.py
"""
import json
import os

import numpy as np

F = np.float32


def lj(r2):
    s = 1.0 / r2
    x2 = s * s
    return 4.0 * ((x2 * x2) * x2 - s * (s * s))


def wca(r2):
    rc = 2.0 ** (1.0 / 6.0)
    if r2 < rc * rc:
        return lj(r2) + 1.0
    return 0.0


def philox(c, k):
    M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
    c = list(c)
    k0, k1 = k
    for r in range(10):
        if r:
            k0 = (k0 + W0) & 0xffffffff
            k1 = (k1 + W1) & 0xffffffff
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & 0xffffffff, p1 & 0xffffffff,
             ((p0 >> 32) ^ c[3] ^ k1) & 0xffffffff, p0 & 0xffffffff]
    return c


def u_open(x):
    return (F(x >> 9) + F(0.5)) * F(1.0 / 8388608.0)


def ln_series(x):
    b = int(np.array([x], np.float32).view(np.uint32)[0])
    e = ((b >> 23) & 0xff) - 127
    m = np.array([(b & 0x7fffff) | 0x3f800000], np.uint32).view(np.float32)[0]
    if m > F(1.41421356):
        m = m * F(0.5)
        e += 1
    s = (m - F(1)) / (m + F(1))
    s2 = s * s
    p = F(1 / 11)
    for c in (1 / 9, 1 / 7, 1 / 5, 1 / 3, 1.0):
        p = p * s2 + F(c)
    return F(e) * F(0.693147182) + (s + s) * p


def sincos_q(phi):
    x2 = phi * phi
    ps = F(-1 / 39916800)
    for c in (1 / 362880, -1 / 5040, 1 / 120, -1 / 6, 1.0):
        ps = ps * x2 + F(c)
    pc = F(1 / 479001600)
    for c in (-1 / 3628800, 1 / 40320, -1 / 720, 1 / 24, -0.5, 1.0):
        pc = pc * x2 + F(c)
    return phi * ps, pc


def normal_pair(a, b):
    u1, u2 = u_open(a), u_open(b)
    r = np.sqrt(F(-2.0) * ln_series(u1))
    q4 = u2 * F(4)
    q = int(q4)
    f = q4 - F(q)
    s, c = sincos_q(f * F(1.57079637))
    cs, sn = [(c, s), (-s, c), (-c, -s), (s, -c)][q & 3]
    return r * cs, r * sn


def u53(a, b):
    return float(((a >> 5) << 26) | (b >> 6)) * (1.0 / 9007199254740992.0)


def draws(system, n, seed, walker, t):
    key = (walker, seed & 0xffffffff)
    shi = seed >> 32
    A = philox((t & 0xffffffff, t >> 32, 0, shi), key)
    if system == 0:
        return [(A[0] * n) >> 32, (A[1] * n) >> 32], [0.0, 0.0, 0.0], u53(A[2], A[3])
    B = philox((t & 0xffffffff, t >> 32, 1, shi), key)
    g0, g1 = normal_pair(A[1], A[2])
    g2, _ = normal_pair(A[3], B[0])
    return [(A[0] * n) >> 32, 0], [float(g0), float(g1), float(g2)], u53(B[1], B[2])


def ising_exact(L):
    N = L * L
    counts = {}
    idx = np.arange(N)
    i, j = idx % L, idx // L
    right = ((i + 1) % L) + j * L
    down = i + ((j + 1) % L) * L
    for state in range(2 ** N):
        s = np.array([1 if (state >> k) & 1 else -1 for k in range(N)])
        e = int((s * (s[right] + s[down])).sum())
        counts[e] = counts.get(e, 0) + 1
    E = sorted(counts)
    return E, [float(np.log(counts[e])) for e in E]


def cv(T, E, S):
    C = []
    for t in T:
        b = S - E / t
        P = np.exp(b - b.max())
        P = P / P.sum()
        U = (E * P).sum()
        C.append(float(((E - U) ** 2 * P).sum() / t ** 2))
    return C


def main():
    r2s = [0.64, 0.81, 1.0, 1.2599210498948732, 1.5, 2.25, 6.25, 0.9, 1.1]
    out = {
        "lj_potential": [[r2, lj(r2)] for r2 in r2s],
        "wca_potential": [[r2, wca(r2)] for r2 in r2s],
        "draws": [],
    }
    for (system, n, seed, walker, t) in [(1, 31, 0, 0, 1), (1, 31, 7, 4095, 123456789),
                                         (1, 1024, 2**40 + 3, 17, 2**33 + 5), (0, 32, 1, 0, 1),
                                         (0, 32, 9, 3, 99999), (1, 38, 5, 8191, 77)]:
        idx, g, u = draws(system, n, seed, walker, t)
        out["draws"].append(dict(system=system, n=n, seed=seed, walker=walker, t=t,
                                 idx=[int(x) for x in idx], g=g, u=u))
    E, lng = ising_exact(4)
    out["ising4_exact"] = dict(E=E, lng=lng)
    rng = np.random.default_rng(11)
    Ec = np.sort(rng.uniform(-134, 0, 200))
    Sc = rng.uniform(0, 60, 200)
    Tc = np.linspace(0.05, 0.5, 25)
    out["cv"] = dict(T=Tc.tolist(), E=Ec.tolist(), S=Sc.tolist(), C=cv(Tc, Ec, Sc))
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
