/* Oracle: C++ restatement of the reference's FP64 CPU MPIDForce (test infrastructure
 * only -- loaded by tests/, __graft_entry__.smoke() and bench.py's CPU baseline, never
 * by the product).
 *
 * It follows the steps of MPIDReferenceForce::calculateForceAndEnergy
 * (platforms/reference/src/SimTKReference/MPIDReferenceForce.cpp:2238-2270) for PME and
 * no-cutoff systems, with two implementation choices of its own:
 *   - pair interactions are written with Cartesian derivative tensors of the radial
 *     kernels (a McMurchie-Davidson style recursion) instead of the reference's
 *     pair-axis frame, so this oracle is an independent formulation;
 *   - real-space pairs come from a cell list (the reference loops over all N^2 pairs)
 *     and loops run in parallel with OpenMP.
 * The PME order may be 5 or 6 (the reference fixes 6, MPIDReferenceForce.cpp:2539).
 * Z-only torques map through the frame's lab axis, as the reference CUDA platform does
 * (platforms/cuda/src/kernels/multipoles.cu:527-533).
 */
#include "mpid_oracle.h"
#include "ref_shim/fftpack.h"

#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

const double ELECTRIC = 138.935455846;  // MPIDReferenceForce.cpp:38
const double SQRT_PI_REF = 1.77245385091;  // MPIDReferenceForce.cpp:2541
const double DEBYE = 48.033324;            // MPIDReferenceForce.cpp:47

// ---------------------------------------------------------------------------
// Symmetric Cartesian tensors of rank 0..3 stored by unique component (t, u, v) =
// number of x, y, z indices.  20 components in order of rank.
struct Comp {
    int t, u, v, rank;
    double w;  // multinomial weight rank!/(t!u!v!)
};
const Comp COMPS[20] = {
    {0, 0, 0, 0, 1},  {1, 0, 0, 1, 1},  {0, 1, 0, 1, 1},  {0, 0, 1, 1, 1},  {2, 0, 0, 2, 1},
    {1, 1, 0, 2, 2},  {1, 0, 1, 2, 2},  {0, 2, 0, 2, 1},  {0, 1, 1, 2, 2},  {0, 0, 2, 2, 1},
    {3, 0, 0, 3, 1},  {2, 1, 0, 3, 3},  {2, 0, 1, 3, 3},  {1, 2, 0, 3, 3},  {1, 1, 1, 3, 6},
    {1, 0, 2, 3, 3},  {0, 3, 0, 3, 1},  {0, 2, 1, 3, 3},  {0, 1, 2, 3, 3},  {0, 0, 3, 3, 1},
};
int comp_of(int t, int u, int v) {
    for (int c = 0; c < 20; ++c)
        if (COMPS[c].t == t && COMPS[c].u == u && COMPS[c].v == v) return c;
    return -1;
}
// component index of a full index tuple
int comp_of_indices(const int* idx, int m) {
    int c[3] = {0, 0, 0};
    for (int k = 0; k < m; ++k) c[idx[k]]++;
    return comp_of(c[0], c[1], c[2]);
}

// ---------------------------------------------------------------------------
// Radial kernels.  g_n = ((1/r) d/dr)^n f.  Bare 1/r: g_n = (-1)^n (2n-1)!!/r^(2n+1).
void bare_g(double r, int nmax, double* g) {
    double ri = 1.0 / r, ri2 = ri * ri;
    g[0] = ri;
    for (int n = 1; n <= nmax; ++n) g[n] = -(2 * n - 1) * g[n - 1] * ri2;
}
// erfc(alpha r)/r: b_n recursion of MPIDReferenceForce.cpp:2840-2857 (b_n = (-1)^n g_n)
void erfc_g(double r, double alpha, int nmax, double* g) {
    double ar = alpha * r, ex = std::exp(-ar * ar), r2 = r * r;
    double b = std::erfc(ar) / r;
    g[0] = b;
    double c = 2.0 * alpha / SQRT_PI_REF * ex;  // (2 alpha^2)^n/(alpha sqrt pi) exp, n = 1
    for (int n = 1; n <= nmax; ++n) {
        b = ((2 * n - 1) * b + c) / r2;
        c *= 2.0 * alpha * alpha;
        g[n] = (n & 1) ? -b : b;
    }
}
// Thole screening lambda_(2n+1) for the damped MPID potential (1-(1+s/2)e^-s)/r,
// s = a r/(d_i d_j); lambda_3..lambda_11 as MPIDReferenceForce.cpp:818-833 and the
// pair-kernel factors of :4509-4523 imply.
const double THOLE_P[6][7] = {
    {1, 0.5, 0, 0, 0, 0, 0},
    {1, 1, 0.5, 0, 0, 0, 0},
    {1, 1, 0.5, 1.0 / 6, 0, 0, 0},
    {1, 1, 0.5, 1.0 / 6, 1.0 / 30, 0, 0},
    {1, 1, 0.5, 1.0 / 6, 4.0 / 105, 1.0 / 210, 0},
    {1, 1, 0.5, 1.0 / 6, 5.0 / 126, 2.0 / 315, 1.0 / 1890},
};
void thole_lambda(double s, int nmax, double* lam) {
    double e = std::exp(-s);
    for (int n = 0; n <= nmax; ++n) {
        double p = 0, sk = 1;
        for (int k = 0; k < 7; ++k) { p += THOLE_P[n][k] * sk; sk *= s; }
        lam[n] = 1.0 - e * p;
    }
}
// d lambda / ds = e^-s (P_n(s) - P_n'(s)), for the polarisability and Thole gradients.
void thole_lambda_ds(double s, int nmax, double* dl) {
    double e = std::exp(-s);
    for (int n = 0; n <= nmax; ++n) {
        double p = 0, sk = 1;
        for (int k = 0; k < 7; ++k) {
            const double next = k + 1 < 7 ? (k + 1) * THOLE_P[n][k + 1] : 0.0;
            p += (THOLE_P[n][k] - next) * sk;
            sk *= s;
        }
        dl[n] = e * p;
    }
}

// Derivative tensor D(t,u,v) = d^t/dx^t d^u/dy^u d^v/dz^v f(|R|) for t+u+v <= L from
// g_n, by R^(n)_(t+1,u,v) = t R^(n+1)_(t-1,u,v) + X R^(n+1)_(t,u,v) (and y, z).
struct DTensor {
    int L;
    double d[9][9][9];
    double operator()(int t, int u, int v) const { return d[t][u][v]; }
};
void derivative_tensor(const double* R, const double* g, int L, DTensor& out) {
    // work[n][t][u][v]
    static thread_local double work[9][9][9][9];
    for (int n = 0; n <= L; ++n) work[n][0][0][0] = g[n];
    for (int n = L - 1; n >= 0; --n)
        for (int v = 0; v + n < L; ++v) {
            // fill (0,0,v+1) at level n from level n+1
            double val = R[2] * work[n + 1][0][0][v];
            if (v > 0) val += v * work[n + 1][0][0][v - 1];
            work[n][0][0][v + 1] = val;
        }
    for (int n = L - 1; n >= 0; --n)
        for (int tot = 0; tot + n < L; ++tot)
            for (int u = 0; u <= tot; ++u) {
                int v = tot - u;
                double val = R[1] * work[n + 1][0][u][v];
                if (u > 0) val += u * work[n + 1][0][u - 1][v];
                work[n][0][u + 1][v] = val;
            }
    for (int n = L - 1; n >= 0; --n)
        for (int tot = 0; tot + n < L; ++tot)
            for (int t = 0; t <= tot; ++t)
                for (int u = 0; t + u <= tot; ++u) {
                    int v = tot - t - u;
                    double val = R[0] * work[n + 1][t][u][v];
                    if (t > 0) val += t * work[n + 1][t - 1][u][v];
                    work[n][t + 1][u][v] = val;
                }
    out.L = L;
    for (int t = 0; t <= L; ++t)
        for (int u = 0; t + u <= L; ++u)
            for (int v = 0; t + u + v <= L; ++v) out.d[t][u][v] = work[0][t][u][v];
}

// ---------------------------------------------------------------------------
struct Atom {
    double q, d[3], Q[3][3], O[3][3][3];
    double M[20];       // unique-component multipole (q, d, Q, O)
    double alpha[3][3]; // lab polarisability
    double thole, damp;
    bool aniso;
    double sph[16];     // spherical moments (self energy)
};

struct Port {
    const mpid_oracle_input* in;
    int n;
    bool pme;
    int order;
    double box[3], recip[3];
    double V[9];        // box rows a, b, c (reduced form; rectangular: diagonal)
    double R[3][3];     // reciprocal vectors as MPIDReferenceForce.cpp:2627-2632 stores them
    bool tri = false;
    double A[3][3];  // frac_j = sum_i A[j][i] x_i
    std::vector<Atom> at;
    std::vector<std::map<int, double>> scale;  // per lower-index atom
    std::vector<std::pair<int, int>> pairs;
    // PME
    int nx, ny, nz;
    std::vector<double> modx, mody, modz;
    std::vector<std::array<int, 3>> igrid;
    std::vector<std::vector<double>> th[3];  // per atom: [5][order]
    std::vector<double> phiP, phiD;          // 35 per atom
    int nthreads;

    double getscale(int i, int j) const {
        int a = std::min(i, j), b = std::max(i, j);
        auto it = scale[a].find(b);
        return it == scale[a].end() ? 1.0 : it->second;
    }
    // minimum image: c, then b, then a (MPIDReferenceForce.cpp:2673-2675)
    void minimg(double* d) const {
        if (!pme) return;
        for (int k = 2; k >= 0; --k) {
            const double s = std::floor(d[k] / box[k] + 0.5);
            for (int q = 0; q <= k; ++q) d[q] -= s * V[3 * k + q];
        }
    }

    // --- frames (MPIDReferenceForce.cpp:357-563) ---
    static double norm3(double* v) {
        double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (r > 0) { v[0] /= r; v[1] /= r; v[2] /= r; }
        return r;
    }
    void frame(int i, double R[3][3]) const {
        int ax = in->axis_type[i];
        if (ax == 5) {
            for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) R[a][b] = a == b;
            return;
        }
        const double* P = in->pos;
        const double* pI = P + 3 * i;
        const double* pZ = P + 3 * in->atom_z[i];
        double vz[3], vx[3], vy[3];
        for (int k = 0; k < 3; ++k) vz[k] = pZ[k] - pI[k];
        norm3(vz);
        if (ax == 4) {
            bool ux = std::fabs(vz[0]) < 0.866;
            vx[0] = ux; vx[1] = !ux; vx[2] = 0;
        } else {
            const double* pX = P + 3 * in->atom_x[i];
            for (int k = 0; k < 3; ++k) vx[k] = pX[k] - pI[k];
            if (ax == 1) {
                norm3(vx);
                for (int k = 0; k < 3; ++k) vz[k] += vx[k];
                norm3(vz);
            } else if (ax == 2 || ax == 3) {
                const double* pY = P + 3 * in->atom_y[i];
                norm3(vx);
                for (int k = 0; k < 3; ++k) vy[k] = pY[k] - pI[k];
                norm3(vy);
                if (ax == 2) {
                    for (int k = 0; k < 3; ++k) vx[k] += vy[k];
                    norm3(vx);
                } else {
                    for (int k = 0; k < 3; ++k) vz[k] += vx[k] + vy[k];
                    norm3(vz);
                }
            }
        }
        double dt = vz[0] * vx[0] + vz[1] * vx[1] + vz[2] * vx[2];
        for (int k = 0; k < 3; ++k) vx[k] -= dt * vz[k];
        norm3(vx);
        vy[0] = vz[1] * vx[2] - vz[2] * vx[1];
        vy[1] = vz[2] * vx[0] - vz[0] * vx[2];
        vy[2] = vz[0] * vx[1] - vz[1] * vx[0];
        for (int k = 0; k < 3; ++k) { R[0][k] = vx[k]; R[1][k] = vy[k]; R[2][k] = vz[k]; }
    }
    bool chiral(int i) const {
        if (in->axis_type[i] != 0 || in->atom_y[i] < 0) return false;
        const double* P = in->pos;
        const double *pI = P + 3 * i, *pZ = P + 3 * in->atom_z[i], *pX = P + 3 * in->atom_x[i], *pY = P + 3 * in->atom_y[i];
        double a[3], b[3], c[3];
        for (int k = 0; k < 3; ++k) { a[k] = pI[k] - pY[k]; b[k] = pZ[k] - pY[k]; c[k] = pX[k] - pY[k]; }
        double cr[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
        return cr[0] * a[0] + cr[1] * a[1] + cr[2] * a[2] < 0;
    }

    void load_atoms() {
        at.resize(n);
        static const int OCT[10][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {0, 0, 2},
                                      {0, 1, 2}, {1, 1, 2}, {0, 2, 2}, {1, 2, 2}, {2, 2, 2}};
        for (int i = 0; i < n; ++i) {
            Atom& a = at[i];
            double d[3], Q[3][3], O[3][3][3];
            for (int k = 0; k < 3; ++k) d[k] = in->dipole[3 * i + k];
            const double* q = in->quadrupole + 6 * i;  // XX XY YY XZ YZ ZZ
            double Qm[3][3] = {{q[0], q[1], q[3]}, {q[1], q[2], q[4]}, {q[3], q[4], q[5]}};
            std::memcpy(Q, Qm, sizeof(Q));
            for (int c = 0; c < 10; ++c) {
                int idx[3] = {OCT[c][0], OCT[c][1], OCT[c][2]};
                std::sort(idx, idx + 3);
                do { O[idx[0]][idx[1]][idx[2]] = in->octopole[10 * i + c]; } while (std::next_permutation(idx, idx + 3));
            }
            if (chiral(i)) {  // MPIDReferenceForce.cpp:372-380: dipole y, QXY and QYZ only
                d[1] = -d[1];
                Q[0][1] = Q[1][0] = -Q[0][1];
                Q[1][2] = Q[2][1] = -Q[1][2];
            }
            double R[3][3];
            frame(i, R);
            a.q = in->charge[i];
            for (int x = 0; x < 3; ++x) {
                a.d[x] = 0;
                for (int k = 0; k < 3; ++k) a.d[x] += R[k][x] * d[k];
            }
            for (int x = 0; x < 3; ++x)
                for (int y = 0; y < 3; ++y) {
                    double s = 0, al = 0;
                    for (int k = 0; k < 3; ++k) {
                        al += R[k][x] * R[k][y] * in->polarity[3 * i + k];
                        for (int m = 0; m < 3; ++m) s += R[k][x] * R[m][y] * Q[k][m];
                    }
                    a.Q[x][y] = s;
                    a.alpha[x][y] = al;
                }
            for (int x = 0; x < 3; ++x)
                for (int y = 0; y < 3; ++y)
                    for (int z = 0; z < 3; ++z) {
                        double s = 0;
                        for (int k = 0; k < 3; ++k)
                            for (int l = 0; l < 3; ++l)
                                for (int m = 0; m < 3; ++m) s += R[k][x] * R[l][y] * R[m][z] * O[k][l][m];
                        a.O[x][y][z] = s;
                    }
            for (int c = 0; c < 20; ++c) {
                const Comp& C = COMPS[c];
                int idx[3], m = 0;
                for (int k = 0; k < C.t; ++k) idx[m++] = 0;
                for (int k = 0; k < C.u; ++k) idx[m++] = 1;
                for (int k = 0; k < C.v; ++k) idx[m++] = 2;
                a.M[c] = C.rank == 0 ? a.q : C.rank == 1 ? a.d[idx[0]] : C.rank == 2 ? a.Q[idx[0]][idx[1]] : a.O[idx[0]][idx[1]][idx[2]];
            }
            const double* p = in->polarity + 3 * i;
            a.aniso = p[0] != p[1] || p[0] != p[2];
            a.damp = std::pow((p[0] + p[1] + p[2]) / 3.0, 1.0 / 6.0);
            a.thole = in->thole[i];
            // spherical moments for the self energy (MPIDReferenceForce.cpp:318-342)
            const double s3 = std::sqrt(3.0);
            a.sph[0] = a.q;
            a.sph[1] = a.d[2]; a.sph[2] = a.d[0]; a.sph[3] = a.d[1];
            a.sph[4] = 3 * a.Q[2][2];
            a.sph[5] = 2 * s3 * a.Q[0][2];
            a.sph[6] = 2 * s3 * a.Q[1][2];
            a.sph[7] = s3 * (a.Q[0][0] - a.Q[1][1]);
            a.sph[8] = 2 * s3 * a.Q[0][1];
            const double (&o)[3][3][3] = a.O;
            a.sph[9] = 15 * o[2][2][2];
            a.sph[10] = 15 * std::sqrt(1.5) * o[0][2][2];
            a.sph[11] = 15 * std::sqrt(1.5) * o[1][2][2];
            a.sph[12] = 15 * std::sqrt(0.6) * (o[0][0][2] - o[1][1][2]);
            a.sph[13] = 30 * std::sqrt(0.6) * o[0][1][2];
            a.sph[14] = 15 * std::sqrt(0.1) * (o[0][0][0] - 3 * o[0][1][1]);
            a.sph[15] = 15 * std::sqrt(0.1) * (3 * o[0][0][1] - o[1][1][1]);
        }
    }

    void setup_scales() {  // MPIDReferenceForce.cpp:190-225
        scale.assign(n, {});
        const double s[4] = {0.0, 0.0, in->scale14, 1.0};
        for (int i = 0; i < n; ++i)
            for (int t = 0; t < 4; ++t)
                for (int k = in->cov_offsets[8 * i + t]; k < in->cov_offsets[8 * i + t + 1]; ++k) {
                    int j = in->cov_index[k];
                    if (j < i) continue;
                    scale[i][j] = s[t];
                }
    }

    void build_pairs() {
        pairs.clear();
        const double rc = in->cutoff, rc2 = rc * rc;
        int nc[3] = {1, 1, 1};
        if (pme)
            for (int k = 0; k < 3; ++k) nc[k] = std::max(1, (int) std::floor(box[k] / rc));
        if (!pme || tri || nc[0] < 3 || nc[1] < 3 || nc[2] < 3) {  // all pairs (cells assume a rectangular box)
            for (int i = 0; i < n; ++i)
                for (int j = i + 1; j < n; ++j) {
                    double d[3];
                    for (int k = 0; k < 3; ++k) d[k] = in->pos[3 * j + k] - in->pos[3 * i + k];
                    minimg(d);
                    if (!pme || d[0] * d[0] + d[1] * d[1] + d[2] * d[2] <= rc2) pairs.push_back({i, j});
                }
            return;
        }
        std::vector<std::vector<int>> cells(nc[0] * nc[1] * nc[2]);
        std::vector<std::array<int, 3>> cid(n);
        for (int i = 0; i < n; ++i) {
            int c[3];
            for (int k = 0; k < 3; ++k) {
                double x = in->pos[3 * i + k];
                x -= box[k] * std::floor(x / box[k]);
                c[k] = std::min(nc[k] - 1, (int) (x / box[k] * nc[k]));
            }
            cid[i] = {c[0], c[1], c[2]};
            cells[(c[0] * nc[1] + c[1]) * nc[2] + c[2]].push_back(i);
        }
        for (int i = 0; i < n; ++i)
            for (int dx = -1; dx <= 1; ++dx)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dz = -1; dz <= 1; ++dz) {
                        int c0 = (cid[i][0] + dx + nc[0]) % nc[0], c1 = (cid[i][1] + dy + nc[1]) % nc[1],
                            c2 = (cid[i][2] + dz + nc[2]) % nc[2];
                        for (int j : cells[(c0 * nc[1] + c1) * nc[2] + c2]) {
                            if (j <= i) continue;
                            double d[3];
                            for (int k = 0; k < 3; ++k) d[k] = in->pos[3 * j + k] - in->pos[3 * i + k];
                            minimg(d);
                            if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] <= rc2) pairs.push_back({i, j});
                        }
                    }
    }

    // --- radial kernels of a pair ---
    // kind 0 perm (s bare - erf), 1 ind (s thole - erf), 2 uu (thole - erf); g[0..nmax]
    void kernel_g(int kind, int i, int j, double r, double s, int nmax, double* g) const {
        double gb[9], ge[9];
        bare_g(r, nmax, gb);
        double alpha = pme ? in->ewald_alpha : 0.0;
        if (alpha > 0) erfc_g(r, alpha, nmax, ge);
        else for (int k = 0; k <= nmax; ++k) ge[k] = gb[k];
        double lam[9];
        for (int k = 0; k <= nmax; ++k) lam[k] = 1.0;
        if (kind > 0) {
            double dmp = at[i].damp * at[j].damp;
            double a = s == 0.0 ? at[i].thole + at[j].thole : in->default_thole;
            if (dmp > 0) {
                double st = a * r / dmp;
                if (st < 50.0) thole_lambda(st, std::min(nmax, 5), lam);
            }
        }
        // f = scale' * screened(1/r) - erf(alpha r)/r  =  erfc - (1 - scale' lambda) bare
        for (int k = 0; k <= nmax; ++k) {
            double sc = kind == 0 ? s : (kind == 1 ? s * lam[k] : lam[k]);
            g[k] = ge[k] - (1.0 - sc) * gb[k];
        }
    }

    // Derivative of kernel kind 1 or 2 (as kernel_g) with respect to the screening
    // argument st = a r / (d_i d_j), for n = 0..nmax.  Returns false where the pair is
    // not screened (zero polarisability, or st beyond the cut of kernel_g).
    bool kernel_g_ds(int kind, int i, int j, double r, double s, int nmax, double* gd, double& st, double& a) const {
        const double dmp = at[i].damp * at[j].damp;
        a = s == 0.0 ? at[i].thole + at[j].thole : in->default_thole;
        if (!(dmp > 0)) return false;
        st = a * r / dmp;
        if (st >= 50.0) return false;
        double gb[9], dl[9];
        bare_g(r, nmax, gb);
        thole_lambda_ds(st, std::min(nmax, 5), dl);
        for (int k = 0; k <= nmax; ++k) gd[k] = (kind == 1 ? s : 1.0) * dl[k] * gb[k];
        return true;
    }

    // Field at a point displaced by D from a source multipole (unique comps M, ranks <= maxRank):
    // E = -grad phi, phi = sum_n (-1)^n M^(n) . grad^n f.
    static void field_from(const double* M, int maxRank, const DTensor& T, double* E) {
        for (int k = 0; k < 3; ++k) {
            double acc = 0;
            for (int c = 0; c < 20; ++c) {
                const Comp& C = COMPS[c];
                if (C.rank > maxRank) continue;
                int t = C.t + (k == 0), u = C.u + (k == 1), v = C.v + (k == 2);
                acc += ((C.rank & 1) ? -1.0 : 1.0) * C.w * M[c] * T(t, u, v);
            }
            E[k] = -acc;
        }
    }

    // --- PME (MPIDReferenceForce.cpp:2720-3737) ---
    void bsplines() {
        for (int d = 0; d < 3; ++d) th[d].assign(n, std::vector<double>(5 * order, 0.0));
        igrid.resize(n);
        const int gdim[3] = {nx, ny, nz};
        for (int i = 0; i < n; ++i)
            for (int d = 0; d < 3; ++d) {
                const double* x = in->pos + 3 * i;
                double w = x[0] * R[0][d] + x[1] * R[1][d] + x[2] * R[2][d];  // fractional (:3058)
                w -= std::floor(w + 0.5);  // minimum image in [-1/2, 1/2)
                double fr = gdim[d] * (w - (int) (w + 0.5) + 0.5);
                int ifr = (int) std::floor(fr);
                double ww = fr - ifr;
                int ig = ifr - order + 1;
                if (ig < 0) ig += gdim[d];
                igrid[i][d] = ig;
                // M_n(ww + m), m = 0..n-1
                double Am[8][8] = {};
                Am[1][0] = 1.0;
                for (int k = 2; k <= order; ++k)
                    for (int m = 0; m < k; ++m) {
                        double t = ww + m;
                        double left = m < k - 1 ? Am[k - 1][m] : 0.0, right = m >= 1 ? Am[k - 1][m - 1] : 0.0;
                        Am[k][m] = (t * left + (k - t) * right) / (k - 1);
                    }
                static const double binom[5][5] = {{1}, {1, 1}, {1, 2, 1}, {1, 3, 3, 1}, {1, 4, 6, 4, 1}};
                for (int der = 0; der <= 4; ++der)
                    for (int p = 0; p < order; ++p) {
                        int m = order - 1 - p;
                        double acc = 0;
                        for (int j = 0; j <= der; ++j) {
                            int mm = m - j;
                            if (mm >= 0 && mm < order - der) acc += ((j & 1) ? -binom[der][j] : binom[der][j]) * Am[order - der][mm];
                        }
                        th[d][i][der * order + p] = acc;
                    }
            }
    }
    static std::vector<double> moduli(int ord, int N) {
        // M_ord at the integers, DFT modulus, Euler-spline fix and zeta correction
        std::vector<double> prev = {1.0, 0.0, 0.0};
        for (int k = 2; k <= ord; ++k) {
            std::vector<double> nxt(k + 2, 0.0);
            for (int t = 0; t <= k; ++t) {
                double a = t < (int) prev.size() ? prev[t] : 0, b = (t >= 1 && t - 1 < (int) prev.size()) ? prev[t - 1] : 0;
                nxt[t] = (t * a + (k - t) * b) / (k - 1);
            }
            prev = nxt;
        }
        std::vector<double> mod(N);
        for (int i = 0; i < N; ++i) {
            double s1 = 0, s2 = 0;
            for (int k = 0; k < ord && k + 1 <= N - 1; ++k) {
                double arg = 2 * M_PI * i * (k + 1) / N;
                s1 += prev[k + 1] * std::cos(arg);
                s2 += prev[k + 1] * std::sin(arg);
            }
            mod[i] = s1 * s1 + s2 * s2;
        }
        if (mod[0] < 1e-7) mod[0] = 0.5 * mod[1];
        for (int i = 1; i < N - 1; ++i)
            if (mod[i] < 1e-7) mod[i] = 0.5 * (mod[i - 1] + mod[i + 1]);
        if (mod[N - 1] < 1e-7) mod[N - 1] = 0.5 * mod[N - 2];
        for (int i = 0; i < N; ++i) {
            int k = i + 1 > N / 2 ? i - N : i;
            double zeta = 1.0;
            if (k) {
                double f = M_PI * k / N, s1 = 1, s2 = 1;
                for (int j = 1; j <= 50; ++j) {
                    double a = f / (f + M_PI * j), b = f / (f - M_PI * j);
                    s1 += std::pow(a, ord) + std::pow(b, ord);
                    s2 += std::pow(a, 2 * ord) + std::pow(b, 2 * ord);
                }
                zeta = s2 / s1;
            }
            mod[i] *= zeta * zeta;
        }
        return mod;
    }
    // fractional weighted multipole (20 comps, unique order) of a Cartesian multipole
    void frac_multipole(const double* M, double* Mf) const {
        // full tensors from unique comps, transformed index by index with A
        for (int c = 0; c < 20; ++c) {
            const Comp& C = COMPS[c];
            int idx[3], m = 0;
            for (int k = 0; k < C.t; ++k) idx[m++] = 0;
            for (int k = 0; k < C.u; ++k) idx[m++] = 1;
            for (int k = 0; k < C.v; ++k) idx[m++] = 2;
            double acc = 0;
            if (m == 0) acc = M[0];
            else {
                int j[3];
                int lim = 1;
                for (int k = 0; k < m; ++k) lim *= 3;
                for (int e = 0; e < lim; ++e) {
                    int ee = e;
                    double f = 1;
                    for (int k = 0; k < m; ++k) { j[k] = ee % 3; ee /= 3; f *= A[idx[k]][j[k]]; }
                    acc += f * M[comp_of_indices(j, m)];
                }
            }
            Mf[c] = acc * C.w;
        }
    }
    void recip_potential(const std::vector<std::array<double, 20>>& Mf, int ncomp, std::vector<double>& phi) {
        std::vector<t_complex> g((size_t) nx * ny * nz);
        for (int i = 0; i < n; ++i)
            for (int ix = 0; ix < order; ++ix)
                for (int iy = 0; iy < order; ++iy)
                    for (int iz = 0; iz < order; ++iz) {
                        double acc = 0;
                        for (int c = 0; c < ncomp; ++c) {
                            const Comp& C = COMPS[c];
                            acc += Mf[i][c] * th[0][i][C.t * order + ix] * th[1][i][C.u * order + iy] * th[2][i][C.v * order + iz];
                        }
                        int x = (igrid[i][0] + ix) % nx, y = (igrid[i][1] + iy) % ny, z = (igrid[i][2] + iz) % nz;
                        g[((size_t) x * ny + y) * nz + z].re += acc;
                    }
        fftpack_t plan;
        fftpack_init_3d(&plan, nx, ny, nz);
        fftpack_exec_3d(plan, FFTPACK_FORWARD, g.data(), g.data());
        const double vol = box[0] * box[1] * box[2], al = in->ewald_alpha;
#pragma omp parallel for
        for (int kx = 0; kx < nx; ++kx)
            for (int ky = 0; ky < ny; ++ky)
                for (int kz = 0; kz < nz; ++kz) {
                    t_complex& c = g[((size_t) kx * ny + ky) * nz + kz];
                    if (!kx && !ky && !kz) { c.re = c.im = 0; continue; }
                    int mx = kx < (nx + 1) / 2 ? kx : kx - nx, my = ky < (ny + 1) / 2 ? ky : ky - ny, mz = kz < (nz + 1) / 2 ? kz : kz - nz;
                    // m_x a* + m_y b* + m_z c* (:3351-3353)
                    double hx = mx * R[0][0], hy = mx * R[1][0] + my * R[1][1],
                           hz = mx * R[2][0] + my * R[2][1] + mz * R[2][2], m2 = hx * hx + hy * hy + hz * hz;
                    double e = std::exp(-M_PI * M_PI * m2 / (al * al)) / (M_PI * vol * m2 * modx[kx] * mody[ky] * modz[kz]);
                    c.re *= e;
                    c.im *= e;
                }
        fftpack_exec_3d(plan, FFTPACK_BACKWARD, g.data(), g.data());
        fftpack_destroy(plan);
        phi.assign((size_t) 35 * n, 0.0);
#pragma omp parallel for
        for (int i = 0; i < n; ++i)
            for (int ix = 0; ix < order; ++ix)
                for (int iy = 0; iy < order; ++iy)
                    for (int iz = 0; iz < order; ++iz) {
                        int x = (igrid[i][0] + ix) % nx, y = (igrid[i][1] + iy) % ny, z = (igrid[i][2] + iz) % nz;
                        double q = g[((size_t) x * ny + y) * nz + z].re;
                        for (int t = 0; t <= 4; ++t)
                            for (int u = 0; t + u <= 4; ++u)
                                for (int v = 0; t + u + v <= 4; ++v)
                                    phi[35 * i + herm(t, u, v)] += q * th[0][i][t * order + ix] * th[1][i][u * order + iy] * th[2][i][v * order + iz];
                    }
    }
    // 35-term index of (t,u,v), MPIDReferenceForce.cpp:3495-3528 ordering
    static int herm(int t, int u, int v) {
        static int table[5][5][5];
        static bool init = false;
        if (!init) {
            const int ord[35][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1},
                                    {0, 1, 1}, {3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {0, 2, 1}, {1, 0, 2},
                                    {0, 1, 2}, {1, 1, 1}, {4, 0, 0}, {0, 4, 0}, {0, 0, 4}, {3, 1, 0}, {3, 0, 1}, {1, 3, 0}, {0, 3, 1},
                                    {1, 0, 3}, {0, 1, 3}, {2, 2, 0}, {2, 0, 2}, {0, 2, 2}, {2, 1, 1}, {1, 2, 1}, {1, 1, 2}};
            for (int k = 0; k < 35; ++k) table[ord[k][0]][ord[k][1]][ord[k][2]] = k;
            init = true;
        }
        return table[t][u][v];
    }

    // --- fields (MPIDReferenceForce.cpp:2812-2949, 4073-4281) ---
    void fixed_field(std::vector<std::array<double, 3>>& E) {
        E.assign(n, {0, 0, 0});
        if (pme) {
            std::vector<std::array<double, 20>> Mf(n);
            for (int i = 0; i < n; ++i) frac_multipole(at[i].M, Mf[i].data());
            recip_potential(Mf, 20, phiP);
            double self = 4.0 / 3.0 * std::pow(in->ewald_alpha, 3) / SQRT_PI_REF;
            for (int i = 0; i < n; ++i)
                for (int c = 0; c < 3; ++c)
                    E[i][c] = -(A[0][c] * phiP[35 * i + 1] + A[1][c] * phiP[35 * i + 2] + A[2][c] * phiP[35 * i + 3]) + self * at[i].d[c];
        }
        std::vector<std::vector<std::array<double, 3>>> part(nthreads, std::vector<std::array<double, 3>>(n, {0, 0, 0}));
#pragma omp parallel for schedule(dynamic, 256)
        for (long p = 0; p < (long) pairs.size(); ++p) {
            auto& acc = part[omp_get_thread_num()];
            int i = pairs[p].first, j = pairs[p].second;
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = in->pos[3 * j + k] - in->pos[3 * i + k];
            minimg(d);
            double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double s = getscale(i, j);
            double g[9];
            kernel_g(1, i, j, r, s, 4, g);
            DTensor T;
            derivative_tensor(d, g, 4, T);
            // field at J from I: displacement R_J - R_I = d
            double Ej[3], Ei[3];
            field_from(at[i].M, 3, T, Ej);
            // field at I from J: displacement -d -> odd orders flip sign
            DTensor Tm = T;
            for (int t = 0; t <= 4; ++t)
                for (int u = 0; t + u <= 4; ++u)
                    for (int v = 0; t + u + v <= 4; ++v)
                        if ((t + u + v) & 1) Tm.d[t][u][v] = -T.d[t][u][v];
            field_from(at[j].M, 3, Tm, Ei);
            for (int c = 0; c < 3; ++c) { acc[i][c] += Ei[c]; acc[j][c] += Ej[c]; }
        }
        for (auto& pt : part)
            for (int i = 0; i < n; ++i)
                for (int c = 0; c < 3; ++c) E[i][c] += pt[i][c];
    }

    // Field of dipoles mu: real (uu kernel) + reciprocal + self; optional gradient.
    void dipole_field(const std::vector<std::array<double, 3>>& mu, std::vector<std::array<double, 3>>& E,
                      std::vector<std::array<double, 6>>* G, bool keepPhi) {
        E.assign(n, {0, 0, 0});
        if (G) G->assign(n, {0, 0, 0, 0, 0, 0});
        if (pme) {
            std::vector<std::array<double, 20>> Mf(n);
            for (int i = 0; i < n; ++i) {
                Mf[i].fill(0.0);
                for (int j = 0; j < 3; ++j) Mf[i][1 + j] = A[j][0] * mu[i][0] + A[j][1] * mu[i][1] + A[j][2] * mu[i][2];
            }
            std::vector<double> phi;
            recip_potential(Mf, 4, phi);
            double self = 4.0 / 3.0 * std::pow(in->ewald_alpha, 3) / SQRT_PI_REF;
            for (int i = 0; i < n; ++i) {
                for (int c = 0; c < 3; ++c)
                    E[i][c] = -(A[0][c] * phi[35 * i + 1] + A[1][c] * phi[35 * i + 2] + A[2][c] * phi[35 * i + 3]) + self * mu[i][c];
                if (G) {
                    double H[3][3] = {{phi[35 * i + 4], phi[35 * i + 7], phi[35 * i + 8]},
                                      {phi[35 * i + 7], phi[35 * i + 5], phi[35 * i + 9]},
                                      {phi[35 * i + 8], phi[35 * i + 9], phi[35 * i + 6]}};
                    const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
                    for (int q = 0; q < 6; ++q) {
                        double acc = 0;
                        for (int k = 0; k < 3; ++k)
                            for (int l = 0; l < 3; ++l) acc += A[k][ia[q]] * H[k][l] * A[l][ib[q]];
                        (*G)[i][q] -= acc;
                    }
                }
            }
            if (keepPhi) phiD = phi;
        }
        std::vector<std::vector<std::array<double, 9>>> part(nthreads, std::vector<std::array<double, 9>>(n));
        for (auto& pt : part) for (auto& v : pt) v.fill(0.0);
#pragma omp parallel for schedule(dynamic, 256)
        for (long p = 0; p < (long) pairs.size(); ++p) {
            auto& acc = part[omp_get_thread_num()];
            int i = pairs[p].first, j = pairs[p].second;
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = in->pos[3 * j + k] - in->pos[3 * i + k];
            minimg(d);
            double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double s = getscale(i, j);
            double g[9];
            kernel_g(2, i, j, r, s, 3, g);
            // E_a(x) from dipole m at x - src = D: -grad(-m.grad f) = sum_b m_b d_a d_b f
            // (d_a d_b f)(D) = delta_ab g1 + D_a D_b g2 ; gradient adds g2, g3 terms.
            auto add = [&](const double* m, const double* D, double* out, double* grad) {
                double md = m[0] * D[0] + m[1] * D[1] + m[2] * D[2];
                for (int a = 0; a < 3; ++a) out[a] += g[1] * m[a] + g[2] * md * D[a];
                if (grad) {
                    const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
                    for (int q = 0; q < 6; ++q) {
                        int a = ia[q], b = ib[q];
                        grad[q] += g[2] * (m[a] * D[b] + m[b] * D[a] + md * (a == b)) + g[3] * md * D[a] * D[b];
                    }
                }
            };
            double dm[3] = {-d[0], -d[1], -d[2]};
            add(mu[j].data(), dm, &acc[i][0], G ? &acc[i][3] : nullptr);
            add(mu[i].data(), d, &acc[j][0], G ? &acc[j][3] : nullptr);
        }
        for (auto& pt : part)
            for (int i = 0; i < n; ++i) {
                for (int c = 0; c < 3; ++c) E[i][c] += pt[i][c];
                if (G) for (int q = 0; q < 6; ++q) (*G)[i][q] += pt[i][3 + q];
            }
    }

    void amul(int i, const double* v, double* o) const {
        for (int a = 0; a < 3; ++a) o[a] = at[i].alpha[a][0] * v[0] + at[i].alpha[a][1] * v[1] + at[i].alpha[a][2] * v[2];
    }

    // Symmetric eigen-decomposition (cyclic Jacobi) for the DIIS pseudo-inverse.
    static void jacobi(std::vector<std::vector<double>>& a, std::vector<double>& w, std::vector<std::vector<double>>& v) {
        int m = (int) a.size();
        v.assign(m, std::vector<double>(m, 0.0));
        for (int i = 0; i < m; ++i) v[i][i] = 1.0;
        for (int sweep = 0; sweep < 100; ++sweep) {
            double off = 0;
            for (int p = 0; p < m; ++p)
                for (int q = p + 1; q < m; ++q) off += a[p][q] * a[p][q];
            if (off < 1e-300) break;
            for (int p = 0; p < m; ++p)
                for (int q = p + 1; q < m; ++q) {
                    if (std::fabs(a[p][q]) < 1e-300) continue;
                    double th = (a[q][q] - a[p][p]) / (2 * a[p][q]);
                    double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                    double c = 1 / std::sqrt(t * t + 1), s = t * c;
                    for (int k = 0; k < m; ++k) {
                        double akp = a[k][p], akq = a[k][q];
                        a[k][p] = c * akp - s * akq;
                        a[k][q] = s * akp + c * akq;
                    }
                    for (int k = 0; k < m; ++k) {
                        double apk = a[p][k], aqk = a[q][k];
                        a[p][k] = c * apk - s * aqk;
                        a[q][k] = s * apk + c * aqk;
                    }
                    for (int k = 0; k < m; ++k) {
                        double vkp = v[k][p], vkq = v[k][q];
                        v[k][p] = c * vkp - s * vkq;
                        v[k][q] = s * vkp + c * vkq;
                    }
                }
        }
        w.resize(m);
        for (int i = 0; i < m; ++i) w[i] = a[i][i];
    }

    // DIIS coefficients (MPIDReferenceForce.cpp:1254-1291): minimum-norm solution of
    // B c = (-1, 0, ...) by the pseudo-inverse, rank cut as an SVD would make it.
    static std::vector<double> diis(const std::vector<std::vector<std::array<double, 3>>>& errs, int n) {
        int steps = (int) errs.size();
        if (steps == 1) return {1.0};
        int m = steps + 1;
        std::vector<std::vector<double>> B(m, std::vector<double>(m, 0.0));
        for (int i = 0; i < steps; ++i) B[i + 1][0] = B[0][i + 1] = -1;
        for (int i = 0; i < steps; ++i)
            for (int j = i; j < steps; ++j) {
                double s = 0;
                for (int k = 0; k < n; ++k)
                    for (int c = 0; c < 3; ++c) s += errs[i][k][c] * errs[j][k][c];
                B[i + 1][j + 1] = B[j + 1][i + 1] = s;
            }
        std::vector<double> w;
        std::vector<std::vector<double>> V;
        jacobi(B, w, V);
        double smax = 0;
        for (double x : w) smax = std::max(smax, std::fabs(x));
        double tol = m * smax * 2.220446049250313e-16;
        std::vector<double> coef(steps, 0.0);
        for (int i = 1; i < m; ++i) {
            double d = 0;
            for (int j = 0; j < m; ++j)
                if (std::fabs(w[j]) > tol) d -= V[0][j] * V[i][j] / w[j];
            coef[i - 1] = d;
        }
        return coef;
    }

    // --- pair electrostatics (MPIDReferenceForce.cpp:4335-4920 computes the same
    // energy, force and torques in a pair-axis frame) ---
    struct PairOut {
        double e, fJ[3], tI[3], tJ[3];
        double gI[20], gJ[20];  // dE/dM per unique lab component (weighted), both atoms
    };
    static double full(const double* M, const int* idx, int m) { return M[comp_of_indices(idx, m)]; }
    // torque -sum_m m (M^(m) x_1 X^(m)) from unique-comp tensors M and X
    static void torque_of(const double* M, const double* X, double* tau) {
        tau[0] = tau[1] = tau[2] = 0;
        for (int a = 0; a < 3; ++a) {
            int j = (a + 1) % 3, k = (a + 2) % 3;
            double s = 0;
            // rank 1
            s += 1 * (M[1 + j] * X[1 + k] - M[1 + k] * X[1 + j]);
            // rank 2
            for (int l = 0; l < 3; ++l) {
                int ij[2] = {j, l}, ik[2] = {k, l};
                s += 2 * (full(M, ij, 2) * full(X, ik, 2) - full(M, ik, 2) * full(X, ij, 2));
            }
            for (int l = 0; l < 3; ++l)
                for (int p = 0; p < 3; ++p) {
                    int ij[3] = {j, l, p}, ik[3] = {k, l, p};
                    s += 3 * (full(M, ij, 3) * full(X, ik, 3) - full(M, ik, 3) * full(X, ij, 3));
                }
            tau[a] = -s;
        }
    }

    void pair(int i, int j, const double* d, double s, const double* uI, const double* uJ, bool mutual, PairOut& o) const {
        const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        double gP[9], gI[9], gU[9];
        kernel_g(0, i, j, r, s, 7, gP);
        kernel_g(1, i, j, r, s, 5, gI);
        if (mutual) kernel_g(2, i, j, r, s, 3, gU);
        DTensor TP, TI, TU;
        derivative_tensor(d, gP, 7, TP);
        derivative_tensor(d, gI, 5, TI);
        if (mutual) derivative_tensor(d, gU, 3, TU);
        const double* MI = at[i].M;
        const double* MJ = at[j].M;
        double uIc[20] = {0}, uJc[20] = {0};
        for (int k = 0; k < 3; ++k) { uIc[1 + k] = uI[k]; uJc[1 + k] = uJ[k]; }
        double XI[20] = {0}, YJ[20] = {0}, WI[20] = {0}, WJ[20] = {0};
        double Upp = 0, Upi = 0, F[3] = {0, 0, 0};
        for (int a = 0; a < 20; ++a) {
            const Comp& A_ = COMPS[a];
            const double sa = (A_.rank & 1) ? -1.0 : 1.0;
            for (int b = 0; b < 20; ++b) {
                const Comp& B_ = COMPS[b];
                const int t = A_.t + B_.t, u = A_.u + B_.u, v = A_.v + B_.v;
                // permanent-permanent
                const double dP = TP(t, u, v);
                XI[a] += sa * B_.w * MJ[b] * dP;
                YJ[b] += sa * A_.w * MI[a] * dP;
                const double wPP = sa * A_.w * B_.w * MI[a] * MJ[b];
                Upp += wPP * dP;
                F[0] -= wPP * TP(t + 1, u, v);
                F[1] -= wPP * TP(t, u + 1, v);
                F[2] -= wPP * TP(t, u, v + 1);
                if (A_.rank + B_.rank > 4) continue;
                // permanent(I)-induced(J) and induced(I)-permanent(J)
                const double dI = TI(t, u, v);
                if (B_.rank == 1) {
                    XI[a] += sa * uJc[b] * dI;
                    WJ[b] += sa * A_.w * MI[a] * dI;
                    const double w = sa * A_.w * MI[a] * uJc[b];
                    Upi += w * dI;
                    F[0] -= w * TI(t + 1, u, v);
                    F[1] -= w * TI(t, u + 1, v);
                    F[2] -= w * TI(t, u, v + 1);
                }
                if (A_.rank == 1) {
                    YJ[b] += sa * uIc[a] * dI;
                    WI[a] += sa * B_.w * MJ[b] * dI;
                    const double w = sa * B_.w * uIc[a] * MJ[b];
                    Upi += w * dI;
                    F[0] -= w * TI(t + 1, u, v);
                    F[1] -= w * TI(t, u + 1, v);
                    F[2] -= w * TI(t, u, v + 1);
                }
                if (mutual && A_.rank == 1 && B_.rank == 1) {
                    const double dU = TU(t, u, v);
                    WI[a] += sa * uJc[b] * dU;
                    WJ[b] += sa * uIc[a] * dU;
                    const double w = sa * uIc[a] * uJc[b];
                    F[0] -= w * TU(t + 1, u, v);
                    F[1] -= w * TU(t, u + 1, v);
                    F[2] -= w * TU(t, u, v + 1);
                }
            }
        }
        o.e = Upp + 0.5 * Upi;
        for (int k = 0; k < 3; ++k) o.fJ[k] = F[k];
        // at stationary induced dipoles dE/dM = d(Upp + Upi)/dM at fixed dipoles
        for (int a = 0; a < 20; ++a) {
            o.gI[a] = COMPS[a].w * XI[a];
            o.gJ[a] = COMPS[a].w * YJ[a];
        }
        torque_of(MI, XI, o.tI);
        torque_of(MJ, YJ, o.tJ);
        double ti[3], tj[3];
        if (at[i].aniso) {
            torque_of(uIc, WI, ti);
            for (int k = 0; k < 3; ++k) o.tI[k] += ti[k];
        }
        if (at[j].aniso) {
            torque_of(uJc, WJ, tj);
            for (int k = 0; k < 3; ++k) o.tJ[k] += tj[k];
        }
        if (mutual && (at[i].aniso || at[j].aniso)) {
            // The reference's pair-axis torque of anisotropic induced dipoles omits one
            // induced-induced term about the axis (MPIDReferenceForce.cpp:4872-4873);
            // reproduce it with its axis convention (MPIDReferenceForce.cpp:650-684).
            double ez[3] = {d[0] / r, d[1] / r, d[2] / r}, ex[3], ey[3];
            double rho2 = ez[1] * ez[1] + ez[2] * ez[2];
            if (rho2 > 0) {
                double rho = std::sqrt(rho2);
                ex[0] = rho; ex[1] = -ez[0] * ez[1] / rho; ex[2] = -ez[0] * ez[2] / rho;
            } else {
                ex[0] = 0; ex[1] = 1; ex[2] = 0;
            }
            ey[0] = ez[1] * ex[2] - ez[2] * ex[1];
            ey[1] = ez[2] * ex[0] - ez[0] * ex[2];
            ey[2] = ez[0] * ex[1] - ez[1] * ex[0];
            // channel (1,1,m=1) coefficient of the induced-induced kernel: -g1
            const double c1 = -gU[1];
            auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
            if (at[i].aniso) {
                const double t = -c1 * dot(uJ, ex) * dot(uI, ey);
                for (int k = 0; k < 3; ++k) o.tI[k] += t * ez[k];
            }
            if (at[j].aniso) {
                const double t = -c1 * dot(uI, ex) * dot(uJ, ey);
                for (int k = 0; k < 3; ++k) o.tJ[k] += t * ez[k];
            }
        }
    }

    // --- torque -> force (MPIDReferenceForce.cpp:1895-2110) ---
    void torque_to_force(int i, const double* tq, std::vector<std::array<double, 3>>& F) const {
        const int ax = in->axis_type[i];
        if (ax == 5) return;
        const double* P = in->pos;
        const int iz = in->atom_z[i], ix = in->atom_x[i], iy = in->atom_y[i];
        auto cross = [](const double* a, const double* b, double* c) {
            c[0] = a[1] * b[2] - a[2] * b[1];
            c[1] = a[2] * b[0] - a[0] * b[2];
            c[2] = a[0] * b[1] - a[1] * b[0];
        };
        auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
        double u[3], v[3], w[3];
        for (int k = 0; k < 3; ++k) u[k] = P[3 * iz + k] - P[3 * i + k];
        double nu = norm3(u);
        if (ax == 4) {
            bool ux = std::fabs(u[0]) < 0.866;
            v[0] = ux; v[1] = !ux; v[2] = 0;
        } else
            for (int k = 0; k < 3; ++k) v[k] = P[3 * ix + k] - P[3 * i + k];
        double nv = norm3(v);
        if (iy >= 0 && (ax == 2 || ax == 3))
            for (int k = 0; k < 3; ++k) w[k] = P[3 * iy + k] - P[3 * i + k];
        else
            cross(u, v, w);
        double nw = norm3(w);
        double uv[3], uw[3], vw[3];
        cross(v, u, uv); norm3(uv);
        cross(w, u, uw); norm3(uw);
        cross(w, v, vw); norm3(vw);
        double cuv = dot(u, v), suv = std::sqrt(1 - cuv * cuv);
        double cuw = dot(u, w), suw = std::sqrt(1 - cuw * cuw);
        double cvw = dot(v, w), svw = std::sqrt(1 - cvw * cvw);
        double dU = -dot(u, tq), dV = -dot(v, tq), dW = -dot(w, tq);
        if (ax == 0 || ax == 1) {
            double f1 = dV / (nu * suv), f2 = dW / nu, f3 = -dU / (nv * suv), f4 = 0;
            if (ax == 1) { f2 *= 0.5; f4 = 0.5 * dW / nv; }
            for (int k = 0; k < 3; ++k) {
                double fu = uv[k] * f1 + f2 * uw[k], fv = uv[k] * f3 + f4 * vw[k];
                F[iz][k] -= fu;
                F[ix][k] -= fv;
                F[i][k] += fu + fv;
            }
        } else if (ax == 2) {
            double rr[3] = {v[0] + w[0], v[1] + w[1], v[2] + w[2]}, ss[3];
            cross(u, rr, ss);
            norm3(rr);
            norm3(ss);
            double ur[3], us[3];
            cross(rr, u, ur); norm3(ur);
            cross(ss, u, us); norm3(us);
            double cur = dot(u, rr), sur = std::sqrt(1 - cur * cur);
            double cvs = dot(v, ss), svs = std::sqrt(1 - cvs * cvs);
            double cws = dot(w, ss), sws = std::sqrt(1 - cws * cws);
            double t1[3], t2[3];
            for (int k = 0; k < 3; ++k) { t1[k] = v[k] - ss[k] * cvs; t2[k] = w[k] - ss[k] * cws; }
            norm3(t1);
            norm3(t2);
            double c1 = dot(u, t1), s1 = std::sqrt(1 - c1 * c1), c2 = dot(u, t2), s2 = std::sqrt(1 - c2 * c2);
            double dR = -dot(rr, tq), dS = -dot(ss, tq);
            double f1 = dR / (nu * sur), f2 = dS / nu, f3 = dU / (nv * (s1 + s2)), f4 = dU / (nw * (s1 + s2));
            for (int k = 0; k < 3; ++k) {
                double fu = ur[k] * f1 + us[k] * f2, fv = (ss[k] * svs - t1[k] * cvs) * f3, fw = (ss[k] * sws - t2[k] * cws) * f4;
                F[iz][k] -= fu;
                F[ix][k] -= fv;
                F[iy][k] -= fw;
                F[i][k] += fu + fv + fw;
            }
        } else if (ax == 3) {
            for (int k = 0; k < 3; ++k) {
                double du = uw[k] * dW / (nu * suw) + uv[k] * dV / (nu * suv) - uw[k] * dU / (nu * suw) - uv[k] * dU / (nu * suv);
                double dv = vw[k] * dW / (nv * svw) - uv[k] * dU / (nv * suv) - vw[k] * dV / (nv * svw) + uv[k] * dV / (nv * suv);
                double dw = -uw[k] * dU / (nw * suw) - vw[k] * dV / (nw * svw) + uw[k] * dW / (nw * suw) + vw[k] * dW / (nw * svw);
                du /= 3; dv /= 3; dw /= 3;
                F[iz][k] -= du;
                F[ix][k] -= dv;
                if (iy >= 0) F[iy][k] -= dw;
                F[i][k] += du + dv + dw;
            }
        } else if (ax == 4) {
            for (int k = 0; k < 3; ++k) {
                double du = uv[k] * dV / (nu * suv) + uw[k] * dW / nu;
                F[iz][k] -= du;
                F[i][k] += du;
            }
        }
    }

    // Gradient of the Ewald self energy (MPIDReferenceForce.cpp:4283-4318) with respect to
    // the unique lab components of atom i, added to g (fixed induced dipole mu).
    void self_gradient(int i, const double* mu, double* g) const {
        const Atom& a = at[i];
        const double al = in->ewald_alpha, a2 = al * al;
        const double pre = -al * ELECTRIC / SQRT_PI_REF;
        const double s3 = std::sqrt(3.0);
        g[0] += pre * 2 * a.q;
        // the d.mu term is half the permanent-induced self interaction: at stationary
        // dipoles the whole interaction enters the derivative
        for (int k = 0; k < 3; ++k) g[1 + k] += pre * 2.0 / 3.0 * a2 * (2 * a.d[k] + 2 * mu[k]);
        const double cq = pre * 4.0 / 15.0 * a2 * a2, co = pre * 8.0 / 105.0 * a2 * a2 * a2;
        const double* S = a.sph;
        // unique comps 4 xx, 5 xy, 6 xz, 7 yy, 8 yz, 9 zz
        g[4] += cq * 2 * S[7] * s3;
        g[7] -= cq * 2 * S[7] * s3;
        g[9] += cq * 2 * S[4] * 3;
        g[6] += cq * 2 * S[5] * 2 * s3;
        g[8] += cq * 2 * S[6] * 2 * s3;
        g[5] += cq * 2 * S[8] * 2 * s3;
        // unique comps 10 xxx 11 xxy 12 xxz 13 xyy 14 xyz 15 xzz 16 yyy 17 yyz 18 yzz 19 zzz
        const double r15 = std::sqrt(1.5), r06 = std::sqrt(0.6), r01 = std::sqrt(0.1);
        g[19] += co * 2 * S[9] * 15;
        g[15] += co * 2 * S[10] * 15 * r15;
        g[18] += co * 2 * S[11] * 15 * r15;
        g[12] += co * 2 * S[12] * 15 * r06;
        g[17] -= co * 2 * S[12] * 15 * r06;
        g[14] += co * 2 * S[13] * 30 * r06;
        g[10] += co * 2 * S[14] * 15 * r01;
        g[13] -= co * 2 * S[14] * 45 * r01;
        g[11] += co * 2 * S[15] * 45 * r01;
        g[16] -= co * 2 * S[15] * 15 * r01;
    }

    // dE/d(molecular-frame polarisability X Y Z, Thole width) per atom, out[4n].  At
    // stationary dipoles (Mutual, Direct) E = F(mu) with F = U_pp + U_pi + U_uu +
    // 1/2 mu.alpha^-1.mu, U_pi = -mu.E_perm and U_uu = -1/2 mu.T.mu (U_uu absent for
    // Direct), so every derivative is taken at fixed dipoles:
    //  - alpha^-1 term: -1/2 nu_k^2 / p_k^2 with nu = R mu the molecular-frame dipole
    //    (alpha_lab = R^T diag(p) R);
    //  - the screening st = a r / (d_i d_j), d_i = mean(p_i)^(1/6): dst/dp_ik =
    //    -st / (18 mean(p_i)) and, for pairs of covalent scale 0 (whose width is
    //    a_i + a_j), dst/da_i = st / a.
    //
    // Extrapolated (OPT, mu = sum_k cbar_k mu_k, mu_0 = alpha E, mu_(k+1) = alpha T mu_k) is
    // not stationary; its energy -1/2 E.P.E with P = sum_k cbar_k (alpha T)^k alpha
    // (symmetric) gives the explicit adjoint sums
    //   d/dalpha: -1/2 sum_k cbar_k sum_(j=0..k) F_j dalpha F_(k-j), F_0 = E_perm and
    //             F_j = T mu_(j-1) (the field of the previous order);
    //   d/dst (uu kernel): -(g1' S1 + g2' S2) per pair, S1 = sum_(j+m<=n-2)
    //             cbar_(j+m+1) mu_(j,i).mu_(m,l), S2 the same with (mu.d)(mu.d);
    // while the permanent field's screening enters as -mu.dE_perm as for the others.
    void polarization_gradient(const std::vector<std::array<double, 3>>& mu, double* out,
                               const std::vector<std::array<double, 3>>* Efix = nullptr,
                               const std::vector<std::vector<std::array<double, 3>>>* ptMu = nullptr,
                               const std::vector<std::vector<std::array<double, 3>>>* ptE = nullptr,
                               const std::vector<double>* cbar = nullptr) const {
        const int pol = in->polarization_type;
        if (pol == 2 && !(Efix && ptMu && ptE && cbar))
            throw std::runtime_error("the extrapolated polarisation gradient needs the perturbation orders");
        const int nPT = pol == 2 ? (int) cbar->size() : 0;
        std::vector<double> W(n, 0.0), Z(n, 0.0);
        for (const auto& pr : pairs) {
            const int i = pr.first, j = pr.second;
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = in->pos[3 * j + k] - in->pos[3 * i + k];
            minimg(d);
            const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            const double s = getscale(i, j);
            double g[9], st, a;
            if (!kernel_g_ds(1, i, j, r, s, 4, g, st, a)) continue;
            // dU_pi/dst: the permanent field's screening derivative at each dipole
            DTensor T;
            derivative_tensor(d, g, 4, T);
            DTensor Tm = T;
            for (int t = 0; t <= 4; ++t)
                for (int u = 0; t + u <= 4; ++u)
                    for (int v = 0; t + u + v <= 4; ++v)
                        if ((t + u + v) & 1) Tm.d[t][u][v] = -T.d[t][u][v];
            double Ej[3], Ei[3];
            field_from(at[i].M, 3, T, Ej);
            field_from(at[j].M, 3, Tm, Ei);
            double D = 0;
            for (int k = 0; k < 3; ++k) D -= mu[j][k] * Ej[k] + mu[i][k] * Ei[k];
            if (pol == 0) {  // dU_uu/dst = -(g1' mu_i.mu_j + g2' (mu_i.d)(mu_j.d))
                kernel_g_ds(2, i, j, r, s, 2, g, st, a);
                double mm = 0, mi = 0, mj = 0;
                for (int k = 0; k < 3; ++k) {
                    mm += mu[i][k] * mu[j][k];
                    mi += mu[i][k] * d[k];
                    mj += mu[j][k] * d[k];
                }
                D -= g[1] * mm + g[2] * mi * mj;
            } else if (pol == 2 && nPT > 1) {
                kernel_g_ds(2, i, j, r, s, 2, g, st, a);
                double S1 = 0, S2 = 0;
                for (int jo = 0; jo + 1 < nPT; ++jo)
                    for (int mo = 0; jo + mo + 1 < nPT; ++mo) {
                        const auto& ui = (*ptMu)[jo][i];
                        const auto& ul = (*ptMu)[mo][j];
                        double mm = 0, mi = 0, ml = 0;
                        for (int k = 0; k < 3; ++k) {
                            mm += ui[k] * ul[k];
                            mi += ui[k] * d[k];
                            ml += ul[k] * d[k];
                        }
                        S1 += (*cbar)[jo + mo + 1] * mm;
                        S2 += (*cbar)[jo + mo + 1] * mi * ml;
                    }
                D -= g[1] * S1 + g[2] * S2;
            }
            W[i] += st * D;
            W[j] += st * D;
            if (s == 0.0) {
                Z[i] += st * D / a;
                Z[j] += st * D / a;
            }
        }
        for (int i = 0; i < n; ++i) {
            double R[3][3];
            frame(i, R);
            const double* p = in->polarity + 3 * i;
            const double pbar = (p[0] + p[1] + p[2]) / 3.0;
            // molecular-frame fields of the OPT orders: F_0 = E_perm, F_j = T mu_(j-1)
            std::vector<std::array<double, 3>> F(nPT);
            for (int jo = 0; jo < nPT; ++jo) {
                const auto& v = jo == 0 ? (*Efix)[i] : (*ptE)[jo - 1][i];
                for (int k = 0; k < 3; ++k) F[jo][k] = R[k][0] * v[0] + R[k][1] * v[1] + R[k][2] * v[2];
            }
            for (int k = 0; k < 3; ++k) {
                double g = 0.0;
                if (pol == 2) {
                    for (int ko = 0; ko < nPT; ++ko)
                        for (int jo = 0; jo <= ko; ++jo) g -= 0.5 * (*cbar)[ko] * F[jo][k] * F[ko - jo][k];
                } else {
                    const double nu = R[k][0] * mu[i][0] + R[k][1] * mu[i][1] + R[k][2] * mu[i][2];
                    g = p[k] > 0 ? -0.5 * nu * nu / (p[k] * p[k]) : 0.0;
                }
                if (pbar > 0) g -= W[i] / (18.0 * pbar);
                out[4 * i + k] = ELECTRIC * g;
            }
            out[4 * i + 3] = ELECTRIC * Z[i];
        }
    }

    // Unique-lab-component gradient -> molecular-frame API parameters of atom i
    // (charge, dipole X Y Z, quadrupole XX XY YY XZ YZ ZZ, octopole XXX XXY XYY YYY XXZ
    // XYZ YYZ XZZ YZZ ZZZ), through the frame rotation and the chirality flip.
    void local_gradient(int i, const double* g, double* out) const {
        double R[3][3];
        frame(i, R);
        const bool flip = chiral(i);
        // full-entry lab derivatives
        double Gd[3], GQ[3][3], GO[3][3][3];
        for (int x = 0; x < 3; ++x) Gd[x] = g[1 + x];
        for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) {
                int idx[2] = {x, y};
                int c = comp_of_indices(idx, 2);
                GQ[x][y] = g[c] / COMPS[c].w;
                for (int z = 0; z < 3; ++z) {
                    int idx3[3] = {x, y, z};
                    int c3 = comp_of_indices(idx3, 3);
                    GO[x][y][z] = g[c3] / COMPS[c3].w;
                }
            }
        // rotate to the molecular frame: lab = R^T local R
        double Ld[3], LQ[3][3], LO[3][3][3];
        for (int k = 0; k < 3; ++k) {
            Ld[k] = 0;
            for (int x = 0; x < 3; ++x) Ld[k] += R[k][x] * Gd[x];
        }
        for (int k = 0; k < 3; ++k)
            for (int m = 0; m < 3; ++m) {
                double s = 0;
                for (int x = 0; x < 3; ++x)
                    for (int y = 0; y < 3; ++y) s += R[k][x] * R[m][y] * GQ[x][y];
                LQ[k][m] = s;
            }
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l)
                for (int m = 0; m < 3; ++m) {
                    double s = 0;
                    for (int x = 0; x < 3; ++x)
                        for (int y = 0; y < 3; ++y)
                            for (int z = 0; z < 3; ++z) s += R[k][x] * R[l][y] * R[m][z] * GO[x][y][z];
                    LO[k][l][m] = s;
                }
        static const int QAPI[6][2] = {{0, 0}, {0, 1}, {1, 1}, {0, 2}, {1, 2}, {2, 2}};
        static const int OAPI[10][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {0, 0, 2},
                                        {0, 1, 2}, {1, 1, 2}, {0, 2, 2}, {1, 2, 2}, {2, 2, 2}};
        out[0] = g[0];
        for (int k = 0; k < 3; ++k) out[1 + k] = Ld[k];
        for (int c = 0; c < 6; ++c) {
            const int k = QAPI[c][0], m = QAPI[c][1];
            out[4 + c] = (k == m) ? LQ[k][m] : LQ[k][m] + LQ[m][k];
        }
        for (int c = 0; c < 10; ++c) {
            int idx[3] = {OAPI[c][0], OAPI[c][1], OAPI[c][2]};
            std::sort(idx, idx + 3);
            double s = 0;
            do { s += LO[idx[0]][idx[1]][idx[2]]; } while (std::next_permutation(idx, idx + 3));
            out[10 + c] = s;
        }
        if (flip) {  // the flipped parameters enter with the opposite sign
            out[2] = -out[2];
            out[4 + 1] = -out[4 + 1];
            out[4 + 4] = -out[4 + 4];
        }
    }

    int run(mpid_oracle_output* out) {
        n = in->n;
        pme = in->nonbonded_method == 1;
        order = in->pme_order;
        nthreads = omp_get_max_threads();
        if (pme) {
            for (int k = 0; k < 3; ++k) box[k] = in->box[4 * k];
            if (in->box[1] != 0 || in->box[2] != 0 || in->box[5] != 0)
                throw std::runtime_error("port: the box must be in reduced form");
            for (int k = 0; k < 9; ++k) V[k] = in->box[k];
            tri = V[3] != 0 || V[6] != 0 || V[7] != 0;
            const double sc = 1.0 / (V[0] * V[4] * V[8]);
            const double Rr[3][3] = {{V[4] * V[8] * sc, 0, 0},
                                     {-V[3] * V[8] * sc, V[0] * V[8] * sc, 0},
                                     {(V[3] * V[7] - V[4] * V[6]) * sc, -V[0] * V[7] * sc, V[0] * V[4] * sc}};
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) R[i][j] = Rr[i][j];
            double minAllowed = 1.999999 * in->cutoff;
            if (box[0] < minAllowed || box[1] < minAllowed || box[2] < minAllowed)
                throw std::runtime_error("The periodic box size has decreased to less than twice the nonbonded cutoff.");
            nx = in->grid[0]; ny = in->grid[1]; nz = in->grid[2];
            // fractional grid transform a[j][i] = n_j R[i][j] (MPIDReferenceForce.cpp:3081-3084)
            for (int j = 0; j < 3; ++j)
                for (int i = 0; i < 3; ++i) A[j][i] = in->grid[j] * R[i][j];
            modx = moduli(order, nx); mody = moduli(order, ny); modz = moduli(order, nz);
        }
        load_atoms();
        setup_scales();
        build_pairs();
        if (pme) bsplines();
        // fixed field and direct dipoles (MPIDReferenceForce.cpp:1293-1329)
        std::vector<std::array<double, 3>> E, mu(n), mud(n), Ei;
        fixed_field(E);
        for (int i = 0; i < n; ++i) amul(i, E[i].data(), mud[i].data());
        mu = mud;
        const int pol = in->polarization_type;
        int iterations = 0;
        double eps = 0;
        bool converged = true;
        std::vector<std::vector<std::array<double, 3>>> ptMu, ptE;
        std::vector<std::vector<std::array<double, 6>>> ptG;
        std::vector<double> cbar;
        if (pol == 0) {  // DIIS, MPIDReferenceForce.cpp:1182-1252
            std::vector<std::vector<std::array<double, 3>>> prevMu, prevErr;
            converged = false;
            for (int it = 0;; ++it) {
                dipole_field(mu, Ei, nullptr, false);
                std::vector<std::array<double, 3>> newMu(n), err(n);
                double s2 = 0;
                for (int i = 0; i < n; ++i) {
                    double am[3];
                    amul(i, Ei[i].data(), am);
                    for (int c = 0; c < 3; ++c) {
                        newMu[i][c] = mud[i][c] + am[c];
                        err[i][c] = newMu[i][c] - mu[i][c];
                        s2 += err[i][c] * err[i][c];
                    }
                }
                prevMu.push_back(newMu);
                prevErr.push_back(err);
                eps = DEBYE * std::sqrt(s2 / n);
                if (eps < in->mutual_eps) converged = true;
                if (eps < in->mutual_eps || it == in->max_iter) { iterations = it; break; }
                if ((int) prevErr.size() > 20) { prevErr.erase(prevErr.begin()); prevMu.erase(prevMu.begin()); }
                std::vector<double> c = diis(prevErr, n);
                for (int i = 0; i < n; ++i)
                    for (int q = 0; q < 3; ++q) {
                        double v = 0;
                        for (size_t k = 0; k < c.size(); ++k) v += prevMu[k][i][q] * c[k];
                        mu[i][q] = v;
                    }
            }
        } else if (pol == 2) {  // MPIDReferenceForce.cpp:1125-1180
            int nPT = in->n_extrap;
            cbar.assign(nPT, 0.0);
            for (int i = 0; i < nPT; ++i)
                for (int j = i; j < nPT; ++j) cbar[i] += in->extrap_coeffs[j];
            ptMu.push_back(mud);
            for (int m = 1; m < nPT; ++m) {
                std::vector<std::array<double, 6>> G;
                dipole_field(ptMu.back(), Ei, &G, false);
                ptE.push_back(Ei);
                ptG.push_back(G);
                std::vector<std::array<double, 3>> nxt(n);
                for (int i = 0; i < n; ++i) amul(i, Ei[i].data(), nxt[i].data());
                ptMu.push_back(nxt);
            }
            for (int i = 0; i < n; ++i)
                for (int c = 0; c < 3; ++c) {
                    mu[i][c] = 0;
                    for (int k = 0; k < nPT; ++k) mu[i][c] += cbar[k] * ptMu[k][i][c];
                }
        }
        if (!converged) {
            snprintf(out->message, sizeof(out->message), "Induced dipoles did not converge:  iterations=%d eps=%g", iterations, eps);
            out->iterations = iterations;
            out->epsilon = eps;
            out->converged = 0;
            return 1;
        }
        if (pme) dipole_field(mu, Ei, nullptr, true);  // reciprocal potential of the final dipoles
        // --- forces (MPIDReferenceForce.cpp:4922-4986) ---
        std::vector<std::array<double, 3>> F(n, {0, 0, 0}), T(n, {0, 0, 0});
        double energy = 0;
        std::vector<std::vector<std::array<double, 6>>> part(nthreads, std::vector<std::array<double, 6>>(n));
        for (auto& pt : part) for (auto& v : pt) v.fill(0.0);
        std::vector<double> epart(nthreads, 0.0);
        const bool wantGrad = out->grad != nullptr;
        std::vector<std::vector<std::array<double, 20>>> gpart(wantGrad ? nthreads : 0,
                                                               std::vector<std::array<double, 20>>(n));
        for (auto& pt : gpart) for (auto& v : pt) v.fill(0.0);
#pragma omp parallel for schedule(dynamic, 128)
        for (long p = 0; p < (long) pairs.size(); ++p) {
            int tid = omp_get_thread_num();
            int i = pairs[p].first, j = pairs[p].second;
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = in->pos[3 * j + k] - in->pos[3 * i + k];
            minimg(d);
            PairOut o;
            pair(i, j, d, getscale(i, j), mu[i].data(), mu[j].data(), pol == 0, o);
            epart[tid] += ELECTRIC * o.e;
            for (int k = 0; k < 3; ++k) {
                part[tid][j][k] += ELECTRIC * o.fJ[k];
                part[tid][i][k] -= ELECTRIC * o.fJ[k];
                part[tid][i][3 + k] += ELECTRIC * o.tI[k];
                part[tid][j][3 + k] += ELECTRIC * o.tJ[k];
            }
            if (wantGrad)
                for (int c = 0; c < 20; ++c) {
                    gpart[tid][i][c] += ELECTRIC * o.gI[c];
                    gpart[tid][j][c] += ELECTRIC * o.gJ[c];
                }
        }
        std::vector<std::array<double, 20>> G(wantGrad ? n : 0);
        for (auto& g : G) g.fill(0.0);
        for (int t = 0; t < (int) gpart.size(); ++t)
            for (int i = 0; i < n; ++i)
                for (int c = 0; c < 20; ++c) G[i][c] += gpart[t][i][c];
        for (int t = 0; t < nthreads; ++t) {
            energy += epart[t];
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) { F[i][k] += part[t][i][k]; T[i][k] += part[t][i][3 + k]; }
        }
        if (pme) {
            const double al = in->ewald_alpha;
            const double term = 2.0 / 3.0 * ELECTRIC * al * al * al / SQRT_PI_REF;  // self torque, :4320-4333
            double cii = 0, dii = 0, qii = 0, oii = 0;
            for (int i = 0; i < n; ++i) {
                const Atom& a = at[i];
                if (!a.aniso) {
                    double u2[3] = {2 * mu[i][0], 2 * mu[i][1], 2 * mu[i][2]};
                    T[i][0] += term * (a.d[1] * u2[2] - a.d[2] * u2[1]);
                    T[i][1] += term * (a.d[2] * u2[0] - a.d[0] * u2[2]);
                    T[i][2] += term * (a.d[0] * u2[1] - a.d[1] * u2[0]);
                }
                // reciprocal energy, force and torque (:3739-4024), fractional coordinates
                double Mf[20], muf[3];
                frac_multipole(a.M, Mf);
                for (int q = 0; q < 3; ++q) muf[q] = A[q][0] * mu[i][0] + A[q][1] * mu[i][1] + A[q][2] * mu[i][2];
                const double* pp = &phiP[35 * i];
                const double* pd = &phiD[35 * i];
                double ef = 0, ei = 0, f[3] = {0, 0, 0};
                for (int c = 0; c < 20; ++c) {
                    const Comp& C = COMPS[c];
                    ef += Mf[c] * pp[herm(C.t, C.u, C.v)];
                    f[0] += Mf[c] * (pp[herm(C.t + 1, C.u, C.v)] + pd[herm(C.t + 1, C.u, C.v)]);
                    f[1] += Mf[c] * (pp[herm(C.t, C.u + 1, C.v)] + pd[herm(C.t, C.u + 1, C.v)]);
                    f[2] += Mf[c] * (pp[herm(C.t, C.u, C.v + 1)] + pd[herm(C.t, C.u, C.v + 1)]);
                }
                for (int k = 0; k < 3; ++k) {
                    int t = k == 0, u = k == 1, v = k == 2;
                    ei += muf[k] * pp[1 + k];
                    for (int q = 0; q < 3; ++q) {
                        int h = herm(t + (q == 0), u + (q == 1), v + (q == 2));
                        f[q] += muf[k] * (pp[h] + (pol == 0 ? pd[h] : 0.0));
                    }
                }
                energy += 0.5 * ELECTRIC * (ef + ei);
                for (int c = 0; c < 3; ++c) F[i][c] -= ELECTRIC * (A[0][c] * f[0] + A[1][c] * f[1] + A[2][c] * f[2]);
                // torques: multipole (+ anisotropic induced dipole) in the Cartesian potential tensors
                for (int which = 0; which < 2; ++which) {
                    const double* ph = which == 0 ? pp : pd;
                    double X[20];
                    for (int c = 0; c < 20; ++c) {
                        const Comp& C = COMPS[c];
                        // Cartesian derivative d^rank phi along the component's index tuple
                        int idx[3], m = 0;
                        for (int k = 0; k < C.t; ++k) idx[m++] = 0;
                        for (int k = 0; k < C.u; ++k) idx[m++] = 1;
                        for (int k = 0; k < C.v; ++k) idx[m++] = 2;
                        double acc = 0;
                        int lim = 1;
                        for (int k = 0; k < m; ++k) lim *= 3;
                        for (int e = 0; e < lim; ++e) {
                            int ee = e, cnt[3] = {0, 0, 0};
                            double fac = 1;
                            for (int k = 0; k < m; ++k) { int jj = ee % 3; ee /= 3; fac *= A[jj][idx[k]]; cnt[jj]++; }
                            acc += fac * ph[herm(cnt[0], cnt[1], cnt[2])];
                        }
                        X[c] = acc;
                    }
                    if (wantGrad)
                        for (int c = 0; c < 20; ++c) G[i][c] += ELECTRIC * COMPS[c].w * X[c];
                    double M[20];
                    std::memcpy(M, a.M, sizeof(M));
                    bool addInd = which == 0 ? a.aniso : (a.aniso && pol == 0);
                    if (addInd)
                        for (int k = 0; k < 3; ++k) M[1 + k] += mu[i][k];
                    double tau[3];
                    torque_of(M, X, tau);
                    for (int k = 0; k < 3; ++k) T[i][k] += ELECTRIC * tau[k];
                }
                if (wantGrad) self_gradient(i, mu[i].data(), G[i].data());
                cii += a.q * a.q;
                for (int k = 0; k < 3; ++k) dii += a.d[k] * (a.d[k] + mu[i][k]);
                for (int k = 4; k < 9; ++k) qii += a.sph[k] * a.sph[k];
                for (int k = 9; k < 16; ++k) oii += a.sph[k] * a.sph[k];
            }
            const double a2 = al * al;  // self energy, :4283-4318
            energy += -al * ELECTRIC / SQRT_PI_REF * (cii + 2.0 / 3.0 * a2 * dii + 4.0 / 15.0 * a2 * a2 * qii + 8.0 / 105.0 * a2 * a2 * a2 * oii);
        }
        if (out->polgrad) polarization_gradient(mu, out->polgrad, &E, &ptMu, &ptE, &cbar);
        if (pol == 2) {  // OPT response, :4956-4984
            int nPT = in->n_extrap;
            for (int i = 0; i < n; ++i)
                for (int l = 0; l < nPT - 1; ++l)
                    for (int m = 0; m < nPT - 1 - l; ++m) {
                        double p = cbar[l + m + 1];
                        if (std::fabs(p) < 1e-6) continue;
                        const auto& u = ptMu[l][i];
                        const auto& g = ptG[m][i];
                        F[i][0] += p * ELECTRIC * (u[0] * g[0] + u[1] * g[3] + u[2] * g[4]);
                        F[i][1] += p * ELECTRIC * (u[0] * g[3] + u[1] * g[1] + u[2] * g[5]);
                        F[i][2] += p * ELECTRIC * (u[0] * g[4] + u[1] * g[5] + u[2] * g[2]);
                        if (at[i].aniso) {
                            const auto& e = ptE[m][i];
                            T[i][0] += p * ELECTRIC * (u[1] * e[2] - u[2] * e[1]);
                            T[i][1] += p * ELECTRIC * (u[2] * e[0] - u[0] * e[2]);
                            T[i][2] += p * ELECTRIC * (u[0] * e[1] - u[1] * e[0]);
                        }
                    }
        }
        for (int i = 0; i < n; ++i) torque_to_force(i, T[i].data(), F);
        if (wantGrad)
            for (int i = 0; i < n; ++i) local_gradient(i, G[i].data(), out->grad + 20 * i);
        out->energy = energy;
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                out->forces[3 * i + k] = F[i][k];
                if (out->induced) out->induced[3 * i + k] = mu[i][k];
                if (out->labdipoles) out->labdipoles[3 * i + k] = at[i].d[k];
            }
        out->iterations = iterations;
        out->epsilon = eps;
        out->converged = 1;
        return 0;
    }
};

}  // namespace

extern "C" int mpidport_evaluate(const mpid_oracle_input* in, mpid_oracle_output* out) {
    out->message[0] = 0;
    try {
        Port p;
        p.in = in;
        return p.run(out);
    } catch (const std::exception& e) {
        snprintf(out->message, sizeof(out->message), "%s", e.what());
        return 1;
    }
}
