"""Generate qi_tables.cuh: the pair-axis ("quasi-internal", QI) frame algebra of the
real-space multipole pair kernel.

Derivation (independent of how the reference writes it out):

* A pair (I at the origin, J at R = r z) interacts through a radial kernel f(r).  With
  the multipole convention of MPIDForce -- potential of J at x is
      phi_J(x) = sum_n (-1)^n M_J^(n) . grad^n f(|x - R_J|),
  M^(0)=q, M^(1)=mu, M^(2)=Theta, M^(3)=Omega (full symmetric Cartesian tensors) --
  the pair energy is  U = sum_{m,n} (-1)^m M_I^(m) . grad^(m+n) f(R) . M_J^(n).
* Derivatives of f(|x|) at (0,0,r) are written through b_n = (-1)^n ((1/r) d/dr)^n f,
  which for a bare 1/r kernel are b_n = (2n-1)!!/r^(2n+1).
* Moments enter through the real spherical components used by the reference
  (MPIDReferenceForce.cpp:318-342): dipole (z, x, y); Q20 = 3 Tzz, Q21c = 2 sqrt3 Txz,
  Q21s = 2 sqrt3 Tyz, Q22c = sqrt3 (Txx - Tyy), Q22s = 2 sqrt3 Txy; Q30 = 15 Ozzz,
  Q31c = 15 sqrt(3/2) Oxzz, Q31s = 15 sqrt(3/2) Oyzz, Q32c = 15 sqrt(3/5)(Oxxz - Oyyz),
  Q32s = 30 sqrt(3/5) Oxyz, Q33c = 15 sqrt(1/10)(Oxxx - 3 Oxyy),
  Q33s = 15 sqrt(1/10)(3 Oxxy - Oyyy).
  In this frame U couples only components with the same m and parity, so
  U = sum_channels C_c(r) * Q_I[a] Q_J[b].  Each C_c is a short combination of
  r^k b_n; its r-derivative uses d b_n/dr = -r b_(n+1).
* Rotating every moment of one atom about axis u by eps changes its components by
  eps * G_u Q (G_u from the infinitesimal rotation of the Cartesian tensors).  The
  torque intermediates and the transverse pair force follow from rotational invariance.

Run:  python gen_qi_tables.py   (writes qi_tables.cuh next to this file).  Needs sympy.
"""
import itertools
import os

import sympy as sp

r = sp.Symbol("r", positive=True)
NB = 8  # b_0 .. b_7
b = sp.symbols("b0:%d" % NB)

# ---------------------------------------------------------------------------
# Derivatives of f(|x|) at (0, 0, r).  A derivative is kept as {n: P(x,y,z)} meaning
# sum_n P * g_n with g_n = ((1/r)d/dr)^n f, using d/dx_a g_n = x_a g_(n+1).
x, y, z = sp.symbols("x y z")
X = (x, y, z)
_deriv_cache = {(0, 0, 0): {0: sp.Integer(1)}}


def deriv(counts):
    counts = tuple(counts)
    if counts in _deriv_cache:
        return _deriv_cache[counts]
    # peel one derivative off the first non-zero axis
    a = next(i for i in range(3) if counts[i] > 0)
    prev = list(counts)
    prev[a] -= 1
    base = deriv(prev)
    out = {}
    for n, P in base.items():
        dP = sp.diff(P, X[a])
        if dP != 0:
            out[n] = sp.expand(out.get(n, 0) + dP)
        out[n + 1] = sp.expand(out.get(n + 1, 0) + P * X[a])
    out = {n: P for n, P in out.items() if P != 0}
    _deriv_cache[counts] = out
    return out


def deriv_at_axis(counts):
    """Value at (0,0,r) in terms of b_n (g_n = (-1)^n b_n)."""
    val = 0
    for n, P in deriv(counts).items():
        val += P.subs({x: 0, y: 0, z: r}) * (-1) ** n * b[n]
    return sp.expand(val)


# ---------------------------------------------------------------------------
# Spherical components <-> traceless Cartesian tensors.
s3 = sp.sqrt(3)
qs = sp.symbols("q0:16")  # generic spherical component vector
COMP_L = [0, 1, 1, 1, 2, 2, 2, 2, 2, 3, 3, 3, 3, 3, 3, 3]
# (m, parity) per component: parity 0 = cosine-like, 1 = sine-like.
COMP_M = [(0, 0), (0, 0), (1, 0), (1, 1), (0, 0), (1, 0), (1, 1), (2, 0), (2, 1),
          (0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (3, 0), (3, 1)]


def cart_from_sph(Q):
    """Full symmetric Cartesian tensors (q, mu[3], T[3][3], O[3][3][3]) from 16 components."""
    q = Q[0]
    mu = [Q[2], Q[3], Q[1]]  # x, y, z
    Q20, Q21c, Q21s, Q22c, Q22s = Q[4:9]
    Tzz = Q20 / 3
    Txz = Q21c / (2 * s3)
    Tyz = Q21s / (2 * s3)
    Txy = Q22s / (2 * s3)
    dxy = Q22c / s3
    Txx = (-Tzz + dxy) / 2
    Tyy = (-Tzz - dxy) / 2
    T = [[Txx, Txy, Txz], [Txy, Tyy, Tyz], [Txz, Tyz, Tzz]]
    Q30, Q31c, Q31s, Q32c, Q32s, Q33c, Q33s = Q[9:16]
    o = sp.symbols("oxxx oxxy oxxz oxyy oxyz oxzz oyyy oyyz oyzz ozzz")
    oxxx, oxxy, oxxz, oxyy, oxyz, oxzz, oyyy, oyyz, oyzz, ozzz = o
    eqs = [
        sp.Eq(15 * ozzz, Q30),
        sp.Eq(15 * sp.sqrt(sp.Rational(3, 2)) * oxzz, Q31c),
        sp.Eq(15 * sp.sqrt(sp.Rational(3, 2)) * oyzz, Q31s),
        sp.Eq(15 * sp.sqrt(sp.Rational(3, 5)) * (oxxz - oyyz), Q32c),
        sp.Eq(30 * sp.sqrt(sp.Rational(3, 5)) * oxyz, Q32s),
        sp.Eq(15 * sp.sqrt(sp.Rational(1, 10)) * (oxxx - 3 * oxyy), Q33c),
        sp.Eq(15 * sp.sqrt(sp.Rational(1, 10)) * (3 * oxxy - oyyy), Q33s),
        sp.Eq(oxxx + oxyy + oxzz, 0),
        sp.Eq(oxxy + oyyy + oyzz, 0),
        sp.Eq(oxxz + oyyz + ozzz, 0),
    ]
    sol = sp.solve(eqs, o, dict=True)[0]
    val = {k: sp.simplify(sol[k]) for k in o}

    def O(i, j, k):
        idx = tuple(sorted((i, j, k)))
        name = "o" + "".join("xyz"[t] for t in idx)
        return val[sp.Symbol(name)]

    Oc = [[[O(i, j, k) for k in range(3)] for j in range(3)] for i in range(3)]
    return q, mu, T, Oc


def sph_from_cart(mu, T, Oc):
    """16 components from Cartesian tensors (the reference's loadParticleData map)."""
    out = [0] * 16
    out[1], out[2], out[3] = mu[2], mu[0], mu[1]
    out[4] = 3 * T[2][2]
    out[5] = 2 * s3 * T[0][2]
    out[6] = 2 * s3 * T[1][2]
    out[7] = s3 * (T[0][0] - T[1][1])
    out[8] = 2 * s3 * T[0][1]
    out[9] = 15 * Oc[2][2][2]
    out[10] = 15 * sp.sqrt(sp.Rational(3, 2)) * Oc[0][2][2]
    out[11] = 15 * sp.sqrt(sp.Rational(3, 2)) * Oc[1][2][2]
    out[12] = 15 * sp.sqrt(sp.Rational(3, 5)) * (Oc[0][0][2] - Oc[1][1][2])
    out[13] = 30 * sp.sqrt(sp.Rational(3, 5)) * Oc[0][1][2]
    out[14] = 15 * sp.sqrt(sp.Rational(1, 10)) * (Oc[0][0][0] - 3 * Oc[0][1][1])
    out[15] = 15 * sp.sqrt(sp.Rational(1, 10)) * (3 * Oc[0][0][1] - Oc[1][1][1])
    return out


def tensors(Q):
    q, mu, T, Oc = cart_from_sph(Q)
    return [q, mu, T, Oc]


def tensor_entries(t, rank):
    """Iterate (index tuple, value) over a full rank-n tensor."""
    if rank == 0:
        yield (), t
        return
    for idx in itertools.product(range(3), repeat=rank):
        v = t
        for i in idx:
            v = v[i]
        yield idx, v


# ---------------------------------------------------------------------------
# Channel coefficients C(a, b) for spherical components a of I and b of J.
QI = sp.symbols("QI0:16")
QJ = sp.symbols("QJ0:16")


def channel_table(max_l_i=3, max_l_j=3):
    TI = tensors(QI)
    TJ = tensors(QJ)
    U = 0
    for m in range(max_l_i + 1):
        for n in range(max_l_j + 1):
            acc = 0
            for idx_i, vi in tensor_entries(TI[m], m):
                if vi == 0:
                    continue
                for idx_j, vj in tensor_entries(TJ[n], n):
                    if vj == 0:
                        continue
                    counts = [0, 0, 0]
                    for t in idx_i + idx_j:
                        counts[t] += 1
                    d = deriv_at_axis(counts)
                    if d == 0:
                        continue
                    acc += vi * vj * d
            U += (-1) ** m * acc
    U = sp.expand(U)
    table = {}
    for a in range(16):
        if COMP_L[a] > max_l_i:
            continue
        for bb in range(16):
            if COMP_L[bb] > max_l_j:
                continue
            c = sp.simplify(U.coeff(QI[a]).coeff(QJ[bb]))
            if c != 0:
                table[(a, bb)] = sp.expand(c)
    return table


# ---------------------------------------------------------------------------
# Rotation generators: delta Q = eps * G_u Q for an infinitesimal rotation about u.
def generators():
    Qs = sp.symbols("Q0:16")
    q, mu, T, Oc = cart_from_sph(Qs)
    gens = []
    for u in range(3):
        uvec = [1 if k == u else 0 for k in range(3)]
        # W_ik such that (u x v)_i = sum_k W_ik v_k
        W = [[sum(sp.LeviCivita(i, j, k) * uvec[j] for j in range(3)) for k in range(3)] for i in range(3)]
        dmu = [sum(W[i][k] * mu[k] for k in range(3)) for i in range(3)]
        dT = [[sum(W[i][k] * T[k][j] + W[j][k] * T[i][k] for k in range(3)) for j in range(3)] for i in range(3)]
        dO = [[[sum(W[i][m] * Oc[m][j][k] + W[j][m] * Oc[i][m][k] + W[k][m] * Oc[i][j][m] for m in range(3))
                for k in range(3)] for j in range(3)] for i in range(3)]
        dQ = sph_from_cart(dmu, dT, dO)
        G = [[sp.nsimplify(sp.simplify(sp.diff(dQ[a], Qs[c]))) if dQ[a] != 0 else 0 for c in range(16)]
             for a in range(16)]
        gens.append(G)
    return gens


# ---------------------------------------------------------------------------
def cexpr(e):
    """C expression in `real` for a sympy expression linear in b_n with powers of r.

    Each term is emitted as real(coefficient) * rp[k] * b[n] with rp[k] = r^k, so the
    same text compiles for float and double without silent promotion."""
    e = sp.expand(e)
    if e == 0:
        return "real(0)"
    terms = []
    for t in sp.Add.make_args(e):
        coef = sp.Integer(1)
        k = 0
        n = None
        for f in sp.Mul.make_args(t):
            if f in b:
                n = b.index(f)
            elif f == r:
                k += 1
            elif isinstance(f, sp.Pow) and f.base == r:
                k += int(f.exp)
            elif isinstance(f, sp.Pow) and f.base in b:
                raise ValueError(t)
            else:
                coef *= f
        val = float(sp.N(coef, 20))
        factors = []
        if n is not None:
            factors.append("b[%d]" % n)
        if k:
            factors.append("rp[%d]" % k)
        body = "*".join(factors) if factors else "real(1)"
        if val == 1.0:
            terms.append(body)
        elif val == -1.0:
            terms.append("-" + body)
        else:
            terms.append("real(%.17g)*%s" % (val, body))
    s = " + ".join(terms)
    return s.replace("+ -", "- ")


def channel_key(a, bb):
    return (COMP_L[a], COMP_L[bb], COMP_M[a][0])


def emit():
    out = []
    out.append("// Generated by gen_qi_tables.py -- do not edit.  Pair-axis (QI) frame algebra of the")
    out.append("// real-space multipole pair kernel; see the generator for the derivation.")
    out.append("#pragma once")
    out.append("")
    print("deriving permanent-permanent channels ...")
    pp = channel_table(3, 3)
    # Group components into channels (l_i, l_j, m): all (a, b) in a channel share C.
    chans = {}
    for (a, bb), c in pp.items():
        key = channel_key(a, bb)
        chans.setdefault(key, []).append((a, bb, c))
    keys = sorted(chans)
    base = {}
    for key in keys:
        a0, b0, c0 = chans[key][0]
        base[key] = c0
        for a, bb, c in chans[key]:
            ratio = sp.simplify(c / c0)
            assert ratio == 1, (key, a, bb, ratio)
    # Every channel coefficient is linear in b_n: C = sum_n k_n(r) b_n.
    out.append("// Channel list: (l_I, l_J, m).  C[k] multiplies QI[a]*QJ[b] for every (a, b) pair")
    out.append("// of channel k; dC[k] is its r-derivative.  NCH_* counts channels per moment set.")
    chan_index = {key: k for k, key in enumerate(keys)}
    out.append("#define QI_NCH_PP %d" % len(keys))
    out.append("#define QI_CH_DIPOLE_DIPOLE_M1 %d  // channel (1, 1, m=1)" % chan_index[(1, 1, 1)])
    # Channels used by the permanent-induced (dipole on one side) and induced-induced sets.
    pi_keys = [k for k in keys if k[1] == 1]           # J side is a dipole
    ip_keys = [k for k in keys if k[0] == 1]           # I side is a dipole
    uu_keys = [k for k in keys if k[0] == 1 and k[1] == 1]
    out.append("")
    out.append("template <typename real>")
    out.append("__host__ __device__ __forceinline__ void qi_channels_pp(const real* b, const real* rp, real* C, real* dC) {")
    for key in keys:
        c = base[key]
        dc = sp.expand(sp.diff(c.subs({b[n]: sp.Function("B%d" % n)(r) for n in range(NB)}), r))
        # substitute derivative: d/dr b_n = -r b_{n+1}
        for n in range(NB - 1):
            dc = dc.subs(sp.Derivative(sp.Function("B%d" % n)(r), r), -r * b[n + 1])
        for n in range(NB):
            dc = dc.subs(sp.Function("B%d" % n)(r), b[n])
        dc = sp.expand(dc)
        out.append("    C[%d] = %s;   // l=(%d,%d) m=%d" % (chan_index[key], cexpr(c), key[0], key[1], key[2]))
        out.append("    dC[%d] = %s;" % (chan_index[key], cexpr(dc)))
    out.append("}")
    out.append("")
    # Emit (a, b, channel) pair list for contractions.
    pairs = sorted(((a, bb, chan_index[channel_key(a, bb)]) for (a, bb) in pp), key=lambda t: (t[0], t[1]))
    out.append("// (component of I, component of J, channel) for every non-zero coupling.")
    out.append("#define QI_NPAIRS %d" % len(pairs))
    out.append("#define QI_PAIR_LIST(X) \\")
    out.append(" \\\n".join("    X(%d, %d, %d)" % p for p in pairs))
    out.append("")
    # Generators.
    print("deriving rotation generators ...")
    gens = generators()
    for u, name in enumerate("XYZ"):
        out.append("// delta Q = eps * G_%s Q for a rotation by eps about %s (in the pair frame).  Q is the" % (name, name.lower()))
        out.append("// 16-component spherical vector; the dipole block also serves the induced dipoles.")
        out.append("template <typename real>")
        out.append("__host__ __device__ __forceinline__ void qi_rotgen_%s(const real* Q, real* G) {" % name.lower())
        for a in range(16):
            terms = []
            for c in range(16):
                g = gens[u][a][c]
                if g != 0:
                    terms.append("real(%.17g)*Q[%d]" % (float(sp.N(g, 20)), c))
            out.append("    G[%d] = %s;" % (a, " + ".join(terms) if terms else "real(0)"))
        out.append("}")
        out.append("")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "qi_tables.cuh")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", path, "channels:", len(keys), "pairs:", len(pairs))
    for key in keys:
        print(key, base[key])


if __name__ == "__main__":
    emit()
