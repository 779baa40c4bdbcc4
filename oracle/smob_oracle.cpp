// smob_oracle.cpp — FP64 CPU restatement of the reference's sphere mobility path.
// TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); see smob_oracle.h.
//
// Mathematics (restated from first principles, since the reference's SCTL/STKFMM
// dependencies are absent):
//  * Grid: p+1 Gauss-Legendre nodes in cos(theta), north to south, 2p+2 uniform phi,
//    weight a^2 * 2pi/(2p+2) * w_GL; points rotated by the layer quaternion
//    (Sphere/Shexp.cpp:206-271).
//  * Density space: vector spherical harmonics of degree <= p in the body frame,
//    basis {Y r, grad_s Y, r x grad_s Y} with orthonormal Y (no Condon-Shortley phase).
//    G2S is the quadrature L2 projection onto that space, S2G its synthesis.
//  * Self terms on the unit sphere are diagonal in the basis
//    H_n = ((n+1) Y r - grad_s Y)/(2n+1), G_n = n Y r + grad_s Y, X_n = r x grad_s Y:
//      single layer  S:  H -> n/((2n+1)(2n+3)),  G -> (n+1)/((2n-1)(2n+1)),  X -> 1/(2n+1)
//      traction PV   K': H -> 3/(2(2n+1)(2n+3)), G -> -3/(2(2n-1)(2n+1)),   X -> -3/(2(2n+1))
//      one-sided limits: exterior = K' - I/2, interior = K' + I/2.
//    (Derived from 8*pi*u = 2 L[f] - grad(x.L[f]) + grad L[y.f] with L the Laplace
//    single layer; pinned in tests against the general evaluator and direct quadrature.)
//  * Off-surface (near) evaluation uses the same identity with Laplace potentials
//    written in irregular solid harmonics Th_n^m = d_+^m d_z^(n-m)(1/r) / sqrt((n-m)!(n+m)!),
//    whose Cartesian derivatives are index shifts:
//      sigma_ik = (1/4pi)[delta_ik div L - x_j d_i d_k L_j + d_i d_k L_r],
//      u_i      = (1/8pi)[L_i - x_j d_i L_j + d_i L_r].
#include "smob_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using cd = std::complex<double>;
constexpr double PI = 3.14159265358979323846264338327950288;

int g_threads = 0;

inline int ncoef(int p) { return (p + 1) * (p + 2) / 2; }
inline int cidx(int n, int m) { return n * (n + 1) / 2 + m; }

// ---------------------------------------------------------------- quaternion
// q = (w, x, y, z); rotation v -> q v q^-1 (Eigen's Quaternion * Vector3).
inline void qrot(const double* q, const double* v, double* o) {
    if (!q) { o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; return; }
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    // t = 2 (qv x v); o = v + w t + qv x t
    const double tx = 2 * (y * v[2] - z * v[1]);
    const double ty = 2 * (z * v[0] - x * v[2]);
    const double tz = 2 * (x * v[1] - y * v[0]);
    o[0] = v[0] + w * tx + (y * tz - z * ty);
    o[1] = v[1] + w * ty + (z * tx - x * tz);
    o[2] = v[2] + w * tz + (x * ty - y * tx);
}
inline void qinvrot(const double* q, const double* v, double* o) {
    if (!q) { o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; return; }
    const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
    qrot(qc, v, o);
}
// The reference skips rotation when the quaternion maps z to z (Shexp.cpp:449-480);
// such a rotation is about z and still rotates x,y, so the skip is only exact for the
// identity. Here every non-null quaternion is applied.

// ---------------------------------------------------------------- Gauss-Legendre
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(PI * (i + 0.75) / (n + 0.5));
        double dp = 0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1, p1 = 0;
            for (int k = 1; k <= n; ++k) {
                const double p2 = p1;
                p1 = p0;
                p0 = ((2 * k - 1) * z * p1 - (k - 1) * p2) / k;
            }
            dp = n * (z * p0 - p1) / (z * z - 1);
            const double dz = p0 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        {
            double p0 = 1, p1 = 0;
            for (int k = 1; k <= n; ++k) {
                const double p2 = p1;
                p1 = p0;
                p0 = ((2 * k - 1) * z * p1 - (k - 1) * p2) / k;
            }
            dp = n * (z * p0 - p1) / (z * z - 1);
        }
        x[n - 1 - i] = z;  // ascending
        w[n - 1 - i] = 2.0 / ((1 - z * z) * dp * dp);
    }
}

// ---------------------------------------------------------------- tables per order
struct Tables {
    int p, nt, nphi, nc;
    std::vector<double> ct, st, wq;        // per ring (north->south): cos, sin, weight*2pi/nphi (unit sphere)
    std::vector<double> cph, sph;          // per column
    std::vector<double> cosmk, sinmk;      // [m*nphi+k], m<=p+1
    std::vector<double> P, dP, Ps;         // [j*nc + cidx(n,m)]: Pbar, dPbar/dtheta, Pbar/sin
};

void legendre_ring(int p, double t, double s, double* P, double* dP, double* Ps) {
    // orthonormal associated Legendre without Condon-Shortley phase
    std::vector<double> pp(ncoef(p), 0.0);
    pp[cidx(0, 0)] = std::sqrt(1.0 / (4 * PI));
    for (int m = 1; m <= p; ++m) pp[cidx(m, m)] = std::sqrt((2.0 * m + 1) / (2.0 * m)) * s * pp[cidx(m - 1, m - 1)];
    for (int m = 0; m < p; ++m) pp[cidx(m + 1, m)] = std::sqrt(2.0 * m + 3) * t * pp[cidx(m, m)];
    for (int m = 0; m <= p; ++m)
        for (int n = m + 2; n <= p; ++n) {
            const double a = std::sqrt((4.0 * n * n - 1) / (double(n) * n - double(m) * m));
            const double b = std::sqrt((double(n - 1) * (n - 1) - double(m) * m) / (4.0 * (n - 1) * (n - 1) - 1));
            pp[cidx(n, m)] = a * (t * pp[cidx(n - 1, m)] - b * pp[cidx(n - 2, m)]);
        }
    for (int n = 0; n <= p; ++n)
        for (int m = 0; m <= n; ++m) {
            const double prev = (n - 1 >= m) ? pp[cidx(n - 1, m)] : 0.0;
            const double c = (n > 0) ? std::sqrt((double(n) * n - double(m) * m) * (2.0 * n + 1) / (2.0 * n - 1)) : 0.0;
            P[cidx(n, m)] = pp[cidx(n, m)];
            dP[cidx(n, m)] = (n * t * pp[cidx(n, m)] - c * prev) / s;
            Ps[cidx(n, m)] = pp[cidx(n, m)] / s;
        }
}

const Tables& tables(int p) {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<Tables>> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(p);
    if (it != cache.end()) return *it->second;
    auto T = std::make_unique<Tables>();
    T->p = p;
    T->nt = p + 1;
    T->nphi = 2 * p + 2;
    T->nc = ncoef(p);
    std::vector<double> x, w;
    gauss_legendre(p + 1, x, w);
    T->ct.resize(p + 1);
    T->st.resize(p + 1);
    T->wq.resize(p + 1);
    for (int j = 0; j <= p; ++j) {
        T->ct[j] = x[p - j];
        T->st[j] = std::sqrt(1 - x[p - j] * x[p - j]);
        T->wq[j] = w[p - j] * 2 * PI / T->nphi;
    }
    T->cph.resize(T->nphi);
    T->sph.resize(T->nphi);
    for (int k = 0; k < T->nphi; ++k) {
        const double ph = 2 * PI * k / T->nphi;
        T->cph[k] = std::cos(ph);
        T->sph[k] = std::sin(ph);
    }
    T->cosmk.resize((p + 2) * T->nphi);
    T->sinmk.resize((p + 2) * T->nphi);
    for (int m = 0; m <= p + 1; ++m)
        for (int k = 0; k < T->nphi; ++k) {
            // exact integer reduction of m*k modulo nphi keeps the table symmetric
            const long mk = (long(m) * k) % T->nphi;
            const double ph = 2 * PI * mk / T->nphi;
            T->cosmk[m * T->nphi + k] = std::cos(ph);
            T->sinmk[m * T->nphi + k] = std::sin(ph);
        }
    T->P.resize(T->nt * T->nc);
    T->dP.resize(T->nt * T->nc);
    T->Ps.resize(T->nt * T->nc);
    for (int j = 0; j <= p; ++j)
        legendre_ring(p, T->ct[j], T->st[j], &T->P[j * T->nc], &T->dP[j * T->nc], &T->Ps[j * T->nc]);
    auto& ref = *T;
    cache[p] = std::move(T);
    return ref;
}

// ---------------------------------------------------------------- VSH transforms (body frame, unit sphere)
// coeff layout: [radial | gradient | toroidal] blocks of nc complex each (n-major, m=0..n).
void vsh_forward(const Tables& T, const double* g, cd* out) {
    const int p = T.p, nphi = T.nphi, nc = T.nc;
    std::fill(out, out + 3 * nc, cd(0, 0));
    std::vector<cd> Fr(p + 1), Ft(p + 1), Fp(p + 1);
    for (int j = 0; j <= p; ++j) {
        const double ct = T.ct[j], st = T.st[j];
        std::fill(Fr.begin(), Fr.end(), cd(0, 0));
        std::fill(Ft.begin(), Ft.end(), cd(0, 0));
        std::fill(Fp.begin(), Fp.end(), cd(0, 0));
        for (int k = 0; k < nphi; ++k) {
            const double* v = g + 3 * (j * nphi + k);
            const double cp = T.cph[k], sp = T.sph[k];
            const double vr = (v[0] * cp + v[1] * sp) * st + v[2] * ct;
            const double vt = (v[0] * cp + v[1] * sp) * ct - v[2] * st;
            const double vp = -v[0] * sp + v[1] * cp;
            for (int m = 0; m <= p; ++m) {
                const cd e(T.cosmk[m * nphi + k], -T.sinmk[m * nphi + k]);
                Fr[m] += vr * e;
                Ft[m] += vt * e;
                Fp[m] += vp * e;
            }
        }
        const double wq = T.wq[j];
        const double* P = &T.P[j * nc];
        const double* dP = &T.dP[j * nc];
        const double* Ps = &T.Ps[j * nc];
        for (int n = 0; n <= p; ++n) {
            const double inv = n > 0 ? 1.0 / (double(n) * (n + 1)) : 0.0;
            for (int m = 0; m <= n; ++m) {
                const int id = cidx(n, m);
                const cd im(0, m * Ps[id]);
                out[id] += wq * Fr[m] * P[id];
                if (n > 0) {
                    out[nc + id] += wq * inv * (Ft[m] * dP[id] - im * Fp[m]);
                    out[2 * nc + id] += wq * inv * (Fp[m] * dP[id] + im * Ft[m]);
                }
            }
        }
    }
}

// synthesis on table T of coefficients of degree <= pc (pc <= T.p), coefficient block size ncoef(pc)
void vsh_inverse(const Tables& T, int pc, const cd* c, double* g) {
    const int nphi = T.nphi, nc = T.nc, ncc = ncoef(pc);
    std::vector<cd> Gr(pc + 1), Gt(pc + 1), Gp(pc + 1);
    for (int j = 0; j < T.nt; ++j) {
        const double ct = T.ct[j], st = T.st[j];
        const double* P = &T.P[j * nc];
        const double* dP = &T.dP[j * nc];
        const double* Ps = &T.Ps[j * nc];
        for (int m = 0; m <= pc; ++m) {
            cd r(0, 0), t(0, 0), q(0, 0);
            for (int n = m; n <= pc; ++n) {
                const int id = cidx(n, m);
                const cd ar = c[id], as = c[ncc + id], ax = c[2 * ncc + id];
                const cd im(0, m * Ps[id]);
                r += ar * P[id];
                t += as * dP[id] - im * ax;
                q += im * as + ax * dP[id];
            }
            const double eps = m == 0 ? 1.0 : 2.0;
            Gr[m] = eps * r;
            Gt[m] = eps * t;
            Gp[m] = eps * q;
        }
        for (int k = 0; k < nphi; ++k) {
            double vr = 0, vt = 0, vp = 0;
            for (int m = 0; m <= pc; ++m) {
                const double c0 = T.cosmk[m * nphi + k], s0 = T.sinmk[m * nphi + k];
                vr += Gr[m].real() * c0 - Gr[m].imag() * s0;
                vt += Gt[m].real() * c0 - Gt[m].imag() * s0;
                vp += Gp[m].real() * c0 - Gp[m].imag() * s0;
            }
            const double cp = T.cph[k], sp = T.sph[k];
            double* v = g + 3 * (j * nphi + k);
            v[0] = vr * st * cp + vt * ct * cp - vp * sp;
            v[1] = vr * st * sp + vt * ct * sp + vp * cp;
            v[2] = vr * ct - vt * st;
        }
    }
}

// scalar forward transform of degree <= pd on table T (pd <= T.p)
void scalar_forward(const Tables& T, int pd, const double* f, int stride, cd* out) {
    const int nphi = T.nphi, nc = T.nc;
    std::fill(out, out + ncoef(pd), cd(0, 0));
    std::vector<cd> F(pd + 1);
    for (int j = 0; j < T.nt; ++j) {
        std::fill(F.begin(), F.end(), cd(0, 0));
        for (int k = 0; k < nphi; ++k) {
            const double v = f[stride * (j * nphi + k)];
            for (int m = 0; m <= pd; ++m) F[m] += v * cd(T.cosmk[m * nphi + k], -T.sinmk[m * nphi + k]);
        }
        const double* P = &T.P[j * nc];
        for (int n = 0; n <= pd; ++n)
            for (int m = 0; m <= n; ++m) out[cidx(n, m)] += T.wq[j] * F[m] * P[cidx(n, m)];
    }
}

// ---------------------------------------------------------------- self multipliers
// kind: 0 SL, 1 exterior traction, 2 interior traction, 3 PV traction
void self_multiply(int p, const cd* c, int kind, cd* o) {
    const int nc = ncoef(p);
    for (int n = 0; n <= p; ++n) {
        const double dn = n;
        double lh, lg, lx;
        if (kind == 0) {
            lh = dn / ((2 * dn + 1) * (2 * dn + 3));
            lg = (dn + 1) / ((2 * dn - 1) * (2 * dn + 1));
            lx = 1.0 / (2 * dn + 1);
        } else {
            lh = 3.0 / (2 * (2 * dn + 1) * (2 * dn + 3));
            lg = -3.0 / (2 * (2 * dn - 1) * (2 * dn + 1));
            lx = -3.0 / (2 * (2 * dn + 1));
            const double sh = kind == 1 ? -0.5 : (kind == 2 ? 0.5 : 0.0);
            lh += sh;
            lg += sh;
            lx += sh;
        }
        for (int m = 0; m <= n; ++m) {
            const int id = cidx(n, m);
            const cd ar = c[id], as = c[nc + id], ax = c[2 * nc + id];
            const cd h = (ar - dn * as) * lh;
            const cd g = (ar + (dn + 1) * as) / (2 * dn + 1) * lg;
            o[id] = h * ((dn + 1) / (2 * dn + 1)) + dn * g;
            o[nc + id] = n > 0 ? (-h / (2 * dn + 1) + g) : cd(0, 0);
            o[2 * nc + id] = n > 0 ? lx * ax : cd(0, 0);
        }
    }
}

// ---------------------------------------------------------------- irregular solid harmonics
// Th_n^m(x) = d_+^m d_z^(n-m) (1/r) / sqrt((n-m)!(n+m)!), n <= N, 0 <= m <= n.
// Functions are F = Re sum c_nm Th_n^m.
void theta_eval(int N, const double* X, double* re, double* im) {
    const double x = X[0], y = X[1], z = X[2];
    const double r2 = x * x + y * y + z * z;
    const double ir2 = 1.0 / r2;
    re[0] = 1.0 / std::sqrt(r2);
    im[0] = 0;
    for (int m = 1; m <= N; ++m) {
        const int a = cidx(m - 1, m - 1), b = cidx(m, m);
        const double f = -std::sqrt((2.0 * m - 1) / (2.0 * m)) * ir2;
        re[b] = f * (x * re[a] - y * im[a]);
        im[b] = f * (x * im[a] + y * re[a]);
    }
    for (int m = 0; m <= N; ++m) {
        for (int n = m; n < N; ++n) {
            const double d = double(n + 1) * (n + 1) - double(m) * m;
            const double c1 = (2.0 * n + 1) / std::sqrt(d);
            const int i1 = cidx(n, m), i2 = cidx(n + 1, m);
            double pr = 0, pi = 0;
            if (n - 1 >= m) {
                const double c2 = std::sqrt((double(n) * n - double(m) * m) / d);
                pr = c2 * re[cidx(n - 1, m)];
                pi = c2 * im[cidx(n - 1, m)];
            }
            re[i2] = -(c1 * z * re[i1] + pr) * ir2;
            im[i2] = -(c1 * z * im[i1] + pi) * ir2;
        }
    }
}

// derivative along axis (0,1,2) of F = Re sum c Th (degree <= N) -> coefficients of degree <= N+1.
// out must hold ncoef(N+1) and is overwritten.
void dmap(const cd* c, int N, int axis, cd* out) {
    std::fill(out, out + ncoef(N + 1), cd(0, 0));
    const cd I(0, 1);
    for (int n = 0; n <= N; ++n)
        for (int m = 0; m <= n; ++m) {
            const cd cc = c[cidx(n, m)];
            const double ap = std::sqrt(double(n + m + 1) * (n + m + 2));
            const double am = std::sqrt(double(n - m + 1) * (n - m + 2));
            if (axis == 2) {
                out[cidx(n + 1, m)] += cc * std::sqrt(double(n + 1) * (n + 1) - double(m) * m);
            } else if (axis == 0) {
                if (m == 0) {
                    out[cidx(n + 1, 1)] += ap * cc.real();
                } else {
                    out[cidx(n + 1, m + 1)] += 0.5 * ap * cc;
                    out[cidx(n + 1, m - 1)] += -0.5 * am * cc;
                }
            } else {
                if (m == 0) {
                    out[cidx(n + 1, 1)] += -I * (ap * cc.real());
                } else {
                    out[cidx(n + 1, m + 1)] += -0.5 * I * ap * cc;
                    out[cidx(n + 1, m - 1)] += -0.5 * I * am * cc;
                }
            }
        }
}

// Precomputed derivative coefficient sets of one source sphere (unit sphere, body frame).
// Sets (all stored at degree Nd = p+3):
//   0-2 L_j; 3+3j+i d_i L_j; 12+i d_i L_r; 15 div L; 16+6j+s d_i d_k L_j; 34+s d_i d_k L_r
//   with s: (00,11,22,01,02,12) -> 0..5
constexpr int NSETS = 40;
inline int sym(int i, int k) {
    if (i == k) return i;
    if (i > k) std::swap(i, k);
    return (i == 0) ? (k == 1 ? 3 : 4) : 5;
}

struct NearSource {
    int p = 0, Nd = 0, nc = 0;
    std::vector<cd> sets;  // NSETS * nc
    const cd* set(int s) const { return &sets[s * nc]; }
};

void pad_copy(const cd* c, int N, cd* out, int Nout) {
    std::fill(out, out + ncoef(Nout), cd(0, 0));
    for (int n = 0; n <= std::min(N, Nout); ++n)
        for (int m = 0; m <= n; ++m) out[cidx(n, m)] = c[cidx(n, m)];
}

void near_prepare(int p, const cd* coeff_body, NearSource& S) {
    S.p = p;
    S.Nd = p + 3;
    S.nc = ncoef(S.Nd);
    S.sets.assign(NSETS * S.nc, cd(0, 0));
    const int q = p + 1;
    const Tables& Tq = tables(q);
    // Cartesian components on the order-(p+1) grid, then exact scalar transforms of degree p+1
    std::vector<double> g(3 * Tq.nt * Tq.nphi);
    vsh_inverse(Tq, p, coeff_body, g.data());
    std::vector<std::vector<cd>> L(4, std::vector<cd>(ncoef(q), cd(0, 0)));
    for (int k = 0; k < 3; ++k) scalar_forward(Tq, q, g.data() + k, 3, L[k].data());
    for (int n = 0; n <= p; ++n)
        for (int m = 0; m <= n; ++m) L[3][cidx(n, m)] = coeff_body[cidx(n, m)];
    // Laplace single layer in Th basis: c_nm = eps_m (-1)^n sqrt(4pi/(2n+1)) g_nm
    for (int k = 0; k < 4; ++k)
        for (int n = 0; n <= q; ++n)
            for (int m = 0; m <= n; ++m)
                L[k][cidx(n, m)] *= (m == 0 ? 1.0 : 2.0) * ((n & 1) ? -1.0 : 1.0) * std::sqrt(4 * PI / (2.0 * n + 1));
    const int Nd = S.Nd, nc = S.nc;
    std::vector<cd> t1(ncoef(Nd + 1)), t2(ncoef(Nd + 2));
    auto put = [&](int s, const cd* c, int N) { pad_copy(c, N, &S.sets[s * nc], Nd); };
    for (int j = 0; j < 3; ++j) {
        put(j, L[j].data(), q);
        for (int i = 0; i < 3; ++i) {
            dmap(L[j].data(), q, i, t1.data());
            put(3 + 3 * j + i, t1.data(), q + 1);
            for (int k = i; k < 3; ++k) {
                dmap(t1.data(), q + 1, k, t2.data());
                put(16 + 6 * j + sym(i, k), t2.data(), q + 2);
            }
        }
    }
    for (int i = 0; i < 3; ++i) {
        dmap(L[3].data(), q, i, t1.data());
        put(12 + i, t1.data(), q + 1);
        for (int k = i; k < 3; ++k) {
            dmap(t1.data(), q + 1, k, t2.data());
            put(34 + sym(i, k), t2.data(), q + 2);
        }
    }
    for (int j = 0; j < 3; ++j)
        for (int id = 0; id < nc; ++id) S.sets[15 * nc + id] += S.sets[(3 + 3 * j + j) * nc + id];
}

// evaluate u (SL, unit sphere) and t (traction with normal nrm) at body-frame unit-scaled target X
void near_eval_point(const NearSource& S, const double* X, const double* nrm, double* u, double* t,
                     std::vector<double>& re, std::vector<double>& im) {
    const int nc = S.nc;
    theta_eval(S.Nd, X, re.data(), im.data());
    auto val = [&](int s) {
        const cd* c = S.set(s);
        double acc = 0;
        for (int id = 0; id < nc; ++id) acc += c[id].real() * re[id] - c[id].imag() * im[id];
        return acc;
    };
    if (u) {
        double Lv[3], dL[3][3], dR[3];
        for (int j = 0; j < 3; ++j) {
            Lv[j] = val(j);
            for (int i = 0; i < 3; ++i) dL[j][i] = val(3 + 3 * j + i);
        }
        for (int i = 0; i < 3; ++i) dR[i] = val(12 + i);
        for (int i = 0; i < 3; ++i) {
            double a = Lv[i] + dR[i];
            for (int j = 0; j < 3; ++j) a -= X[j] * dL[j][i];
            u[i] = a / (8 * PI);
        }
    }
    if (t) {
        const double D = val(15);
        double H[4][6];
        for (int j = 0; j < 3; ++j)
            for (int s = 0; s < 6; ++s) H[j][s] = val(16 + 6 * j + s);
        for (int s = 0; s < 6; ++s) H[3][s] = val(34 + s);
        for (int i = 0; i < 3; ++i) {
            double a = nrm[i] * D;
            for (int k = 0; k < 3; ++k) {
                double hx = H[3][sym(i, k)];
                for (int j = 0; j < 3; ++j) hx -= X[j] * H[j][sym(i, k)];
                a += nrm[k] * hx;
            }
            t[i] = a / (4 * PI);
        }
    }
}

// ---------------------------------------------------------------- sphere-level helpers (lab frame)
void sh_g2s(int p, const double* q, const double* grid3, cd* coeff) {
    const Tables& T = tables(p);
    const int ng = T.nt * T.nphi;
    std::vector<double> b(3 * ng);
    for (int i = 0; i < ng; ++i) qinvrot(q, grid3 + 3 * i, &b[3 * i]);
    vsh_forward(T, b.data(), coeff);
}
void sh_s2g_body(int p, const cd* coeff, double* grid3) { vsh_inverse(tables(p), p, coeff, grid3); }

int set_threads() {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

// ---------------------------------------------------------------- operator context
struct Ctx {
    int N = 0, M = 0;
    std::vector<double> centers, radii, quats;
    bool has_quat = false;
    std::vector<int> orders, gidx, glen, cidxs, sid;
    double viscosity = 1;
    std::vector<double> coords, norms, weights;
    std::vector<int> ptrg, psrc;  // near pairs sorted by (trg, src)
    const double* q(int i) const { return has_quat ? &quats[4 * i] : nullptr; }
};

void build_pairs(int n, const double* c, const double* r, std::vector<int>& pt, std::vector<int>& ps) {
    pt.clear();
    ps.clear();
    for (int t = 0; t < n; ++t)
        for (int s = 0; s < n; ++s) {
            // MPI/NearInteraction.txx:430-447 with Rad = 1.5*radius (SphereSTKSHOperator.cpp:547)
            double r2 = 0;
            for (int k = 0; k < 3; ++k) {
                const double d = c[3 * s + k] - c[3 * t + k];
                r2 += d * d;
            }
            const double Rn = 1.5 * r[s] + 1.5 * r[t];
            if (r2 > 0 && r2 < Rn * Rn) {
                pt.push_back(t);
                ps.push_back(s);
            }
        }
}

void coeffs_all(const Ctx& C, const double* in, std::vector<std::vector<cd>>& coef) {
    coef.resize(C.N);
#pragma omp parallel for schedule(dynamic) num_threads(set_threads())
    for (int i = 0; i < C.N; ++i) {
        coef[i].assign(3 * ncoef(C.orders[i]), cd(0, 0));
        sh_g2s(C.orders[i], C.q(i), in + 3 * C.gidx[i], coef[i].data());
    }
}

// excl_near: also skip sources on spheres that are near-pair sources of the target's sphere
// (those pairs are then evaluated spectrally only, with no direct subtraction).
void far_field(const Ctx& C, const double* in, double* out, double c, bool trac, bool excl_near = false) {
    const int M = C.M;
    std::vector<char> nb;
    if (excl_near) {
        nb.assign(size_t(C.N) * C.N, 0);
        for (size_t e = 0; e < C.ptrg.size(); ++e) nb[size_t(C.ptrg[e]) * C.N + C.psrc[e]] = 1;
    }
    std::vector<double> f(3 * M);
    for (int i = 0; i < M; ++i)
        for (int k = 0; k < 3; ++k) f[3 * i + k] = in[3 * i + k] * C.weights[i] * c;
    const double* X = C.coords.data();
    const double* Nn = C.norms.data();
#pragma omp parallel for schedule(static) num_threads(set_threads())
    for (int t = 0; t < M; ++t) {
        const double tx = X[3 * t], ty = X[3 * t + 1], tz = X[3 * t + 2];
        const double nx = Nn[3 * t], ny = Nn[3 * t + 1], nz = Nn[3 * t + 2];
        const int st = C.sid[t];
        double ax = 0, ay = 0, az = 0;
        for (int s = 0; s < M; ++s) {
            if (C.sid[s] == st) continue;  // own sphere: replaced by the spectral self term
            if (excl_near && nb[size_t(st) * C.N + C.sid[s]]) continue;
            const double rx = tx - X[3 * s], ry = ty - X[3 * s + 1], rz = tz - X[3 * s + 2];
            const double r2 = rx * rx + ry * ry + rz * rz;
            const double ri = 1.0 / std::sqrt(r2);
            const double fx = f[3 * s], fy = f[3 * s + 1], fz = f[3 * s + 2];
            const double rf = rx * fx + ry * fy + rz * fz;
            if (trac) {
                const double rn = rx * nx + ry * ny + rz * nz;
                const double ri2 = ri * ri;
                const double k = rf * rn * ri2 * ri2 * ri;
                ax += k * rx;
                ay += k * ry;
                az += k * rz;
            } else {
                const double ri3 = ri * ri * ri;
                ax += fx * ri + rf * ri3 * rx;
                ay += fy * ri + rf * ri3 * ry;
                az += fz * ri + rf * ri3 * rz;
            }
        }
        const double pre = trac ? -3.0 / (4 * PI) : 1.0 / (8 * PI);
        out[3 * t] += pre * ax;
        out[3 * t + 1] += pre * ay;
        out[3 * t + 2] += pre * az;
    }
}

void self_terms(const Ctx& C, const std::vector<std::vector<cd>>& coef, double* out, double c, bool trac) {
#pragma omp parallel for schedule(dynamic) num_threads(set_threads())
    for (int i = 0; i < C.N; ++i) {
        const int p = C.orders[i], nc = ncoef(p), ng = C.glen[i];
        std::vector<cd> o(3 * nc);
        self_multiply(p, coef[i].data(), trac ? 3 : 0, o.data());
        std::vector<double> g(3 * ng);
        sh_s2g_body(p, o.data(), g.data());
        const double scale = trac ? c : c * C.radii[i];
        for (int j = 0; j < ng; ++j) {
            double v[3];
            qrot(C.q(i), &g[3 * j], v);
            for (int k = 0; k < 3; ++k) out[3 * (C.gidx[i] + j) + k] += scale * v[k];
        }
    }
}

void near_terms(const Ctx& C, const std::vector<std::vector<cd>>& coef, const double* in, double* out, double c_sl,
                double c_trac) {
    if (C.ptrg.empty()) return;
    // prepare every sphere that is a source of some pair
    std::vector<char> is_src(C.N, 0);
    for (int s : C.psrc) is_src[s] = 1;
    std::vector<NearSource> S(C.N);
#pragma omp parallel for schedule(dynamic) num_threads(set_threads())
    for (int i = 0; i < C.N; ++i)
        if (is_src[i]) near_prepare(C.orders[i], coef[i].data(), S[i]);
    // group pairs by target (pairs sorted by target): each target sphere owned by one thread
    std::vector<int> tstart(C.N + 1, 0);
    for (int t : C.ptrg) tstart[t + 1]++;
    for (int i = 0; i < C.N; ++i) tstart[i + 1] += tstart[i];
#pragma omp parallel num_threads(set_threads())
    {
        std::vector<double> re, im;
#pragma omp for schedule(dynamic)
        for (int t = 0; t < C.N; ++t) {
            for (int e = tstart[t]; e < tstart[t + 1]; ++e) {
                const int s = C.psrc[e];
                const NearSource& src = S[s];
                re.resize(src.nc);
                im.resize(src.nc);
                const double a = C.radii[s];
                const double* qs = C.q(s);
                const int ns = C.glen[s], nt = C.glen[t];
                for (int j = 0; j < nt; ++j) {
                    const int ti = C.gidx[t] + j;
                    double rel[3], xb[3], nb[3], u[3], tr[3], ul[3], tl[3];
                    for (int k = 0; k < 3; ++k) rel[k] = C.coords[3 * ti + k] - C.centers[3 * s + k];
                    qinvrot(qs, rel, xb);
                    for (int k = 0; k < 3; ++k) xb[k] /= a;
                    qinvrot(qs, &C.norms[3 * ti], nb);
                    near_eval_point(src, xb, nb, c_sl != 0 ? u : nullptr, c_trac != 0 ? tr : nullptr, re, im);
                    // direct smooth quadrature over the source grid (what the far field added)
                    double dsl[3] = {0, 0, 0}, dtr[3] = {0, 0, 0};
                    const double* nt3 = &C.norms[3 * ti];
                    for (int sj = 0; sj < ns; ++sj) {
                        const int si = C.gidx[s] + sj;
                        const double rx = C.coords[3 * ti] - C.coords[3 * si];
                        const double ry = C.coords[3 * ti + 1] - C.coords[3 * si + 1];
                        const double rz = C.coords[3 * ti + 2] - C.coords[3 * si + 2];
                        const double w = C.weights[si];
                        const double fx = in[3 * si] * w, fy = in[3 * si + 1] * w, fz = in[3 * si + 2] * w;
                        const double r2 = rx * rx + ry * ry + rz * rz;
                        const double ri = 1.0 / std::sqrt(r2);
                        const double rf = rx * fx + ry * fy + rz * fz;
                        if (c_sl != 0) {
                            const double ri3 = ri * ri * ri;
                            dsl[0] += fx * ri + rf * ri3 * rx;
                            dsl[1] += fy * ri + rf * ri3 * ry;
                            dsl[2] += fz * ri + rf * ri3 * rz;
                        }
                        if (c_trac != 0) {
                            const double rn = rx * nt3[0] + ry * nt3[1] + rz * nt3[2];
                            const double ri2 = ri * ri;
                            const double k = rf * rn * ri2 * ri2 * ri;
                            dtr[0] += k * rx;
                            dtr[1] += k * ry;
                            dtr[2] += k * rz;
                        }
                    }
                    if (c_sl != 0) {
                        qrot(qs, u, ul);
                        for (int k = 0; k < 3; ++k) out[3 * ti + k] += c_sl * (a * ul[k] - dsl[k] / (8 * PI));
                    }
                    if (c_trac != 0) {
                        qrot(qs, tr, tl);
                        for (int k = 0; k < 3; ++k) out[3 * ti + k] += c_trac * (tl[k] + 3.0 / (4 * PI) * dtr[k]);
                    }
                }
            }
        }
    }
}

void apply_p2p(const Ctx& C, const double* in, double* out, double cId, double cSL, double cTrac) {
    std::vector<std::vector<cd>> coef;
    coeffs_all(C, in, coef);
    if (std::fabs(cSL) > 1e-9) {
        far_field(C, in, out, cSL, false);
        self_terms(C, coef, out, cSL, false);
    }
    if (std::fabs(cTrac) > 1e-9) {
        far_field(C, in, out, cTrac, true);
        self_terms(C, coef, out, cTrac, true);
    }
    if (std::fabs(cId) > 1e-9)
        for (int i = 0; i < 3 * C.M; ++i) out[i] += cId * in[i];
    if (std::fabs(cSL) + std::fabs(cTrac) > 1e-9)
        near_terms(C, coef, in, out, std::fabs(cSL) > 1e-9 ? cSL : 0.0, std::fabs(cTrac) > 1e-9 ? cTrac : 0.0);
}

void apply_lop(const Ctx& C, const double* in, double* out, double cLOP) {
    for (int i = 0; i < C.N; ++i) {
        const double a = C.radii[i];
        double A[3] = {0, 0, 0}, B[3] = {0, 0, 0};
        for (int j = 0; j < C.glen[i]; ++j) {
            const int id = C.gidx[i] + j;
            const double w = C.weights[id];
            const double* v = in + 3 * id;
            const double* n = &C.norms[3 * id];
            for (int k = 0; k < 3; ++k) A[k] += w * v[k];
            B[0] += w * a * (n[1] * v[2] - n[2] * v[1]);
            B[1] += w * a * (n[2] * v[0] - n[0] * v[2]);
            B[2] += w * a * (n[0] * v[1] - n[1] * v[0]);
        }
        const double fa = 1.0 / (4 * PI * a * a), fb = 3.0 / (8 * PI * a * a * a * a);
        for (int k = 0; k < 3; ++k) {
            A[k] *= fa;
            B[k] *= fb;
        }
        for (int j = 0; j < C.glen[i]; ++j) {
            const int id = C.gidx[i] + j;
            const double* n = &C.norms[3 * id];
            const double rx = a * n[0], ry = a * n[1], rz = a * n[2];
            out[3 * id] += cLOP * (A[0] + B[1] * rz - B[2] * ry);
            out[3 * id + 1] += cLOP * (A[1] + B[2] * rx - B[0] * rz);
            out[3 * id + 2] += cLOP * (A[2] + B[0] * ry - B[1] * rx);
        }
    }
}

void apply_A(const Ctx& C, const double* x, double* y) {
    // A = 0.5 I + K + L (SphereSTKMobMat.cpp:17 constructs cId=0.5, cSL=0, cTrac=1, cLOP=1)
    std::fill(y, y + 3 * C.M, 0.0);
    apply_p2p(C, x, y, 0.5, 0.0, 1.0);
    apply_lop(C, x, y, 1.0);
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}

// Restarted GMRES with iterated modified Gram-Schmidt (two MGS passes), Givens rotations,
// implicit residual test |g_{j+1}|/|b| < tol, then an explicit residual check at each restart
// (Belos pseudo-block GMRES with "Implicit/Explicit Residual Scaling: Norm of RHS").
int gmres(const Ctx& C, const std::vector<double>& b, std::vector<double>& x, double tol, int m, int maxit,
          int* iters, double* relres) {
    const size_t n = b.size();
    const double bn = std::sqrt(dot(b, b));
    int it = 0;
    if (bn == 0) {
        std::fill(x.begin(), x.end(), 0.0);
        *iters = 0;
        *relres = 0;
        return 0;
    }
    std::vector<double> r(n), w(n);
    auto residual = [&]() {
        bool zero = true;
        for (double v : x)
            if (v != 0) { zero = false; break; }
        if (zero) { r = b; return; }
        apply_A(C, x.data(), w.data());
        for (size_t i = 0; i < n; ++i) r[i] = b[i] - w[i];
    };
    residual();
    double rn = std::sqrt(dot(r, r));
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
    std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    while (true) {
        if (rn / bn < tol || it >= maxit) break;
        for (size_t i = 0; i < n; ++i) V[0][i] = r[i] / rn;
        std::fill(H.begin(), H.end(), 0.0);
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = rn;
        int k = 0;
        for (int j = 0; j < m; ++j) {
            apply_A(C, V[j].data(), w.data());
            ++it;
            for (int pass = 0; pass < 2; ++pass)
                for (int i = 0; i <= j; ++i) {
                    const double h = dot(V[i], w);
                    H[i * m + j] += h;
                    for (size_t l = 0; l < n; ++l) w[l] -= h * V[i][l];
                }
            const double hn = std::sqrt(dot(w, w));
            H[(j + 1) * m + j] = hn;
            if (hn > 0)
                for (size_t l = 0; l < n; ++l) V[j + 1][l] = w[l] / hn;
            for (int i = 0; i < j; ++i) {
                const double a = H[i * m + j], bb = H[(i + 1) * m + j];
                H[i * m + j] = cs[i] * a + sn[i] * bb;
                H[(i + 1) * m + j] = -sn[i] * a + cs[i] * bb;
            }
            {
                const double a = H[j * m + j], bb = H[(j + 1) * m + j];
                const double d = std::hypot(a, bb);
                cs[j] = d > 0 ? a / d : 1.0;
                sn[j] = d > 0 ? bb / d : 0.0;
                H[j * m + j] = d;
                H[(j + 1) * m + j] = 0;
                g[j + 1] = -sn[j] * g[j];
                g[j] = cs[j] * g[j];
            }
            k = j + 1;
            if (std::fabs(g[j + 1]) / bn < tol || it >= maxit || hn == 0) break;
        }
        for (int i = k - 1; i >= 0; --i) {
            double s = g[i];
            for (int l = i + 1; l < k; ++l) s -= H[i * m + l] * y[l];
            y[i] = s / H[i * m + i];
        }
        for (int i = 0; i < k; ++i)
            for (size_t l = 0; l < n; ++l) x[l] += y[i] * V[i][l];
        residual();
        rn = std::sqrt(dot(r, r));
    }
    *iters = it;
    *relres = rn / bn;
    return rn / bn < tol ? 0 : 1;
}

}  // namespace

// ================================================================ C ABI
extern "C" {

int orc_grid_number(int p) { return (p + 1) * (2 * p + 2); }
int orc_spectral_dof(int p) { return 3 * (p + 1) * (p + 2); }
void orc_set_threads(int n) { g_threads = n; }

void orc_gauss_legendre(int n, double* nodes, double* weights) {
    std::vector<double> x, w;
    gauss_legendre(n, x, w);
    std::copy(x.begin(), x.end(), nodes);
    std::copy(w.begin(), w.end(), weights);
}

void orc_sh_grid(int p, double radius, const double* quat, const double* center, double* coords, double* norms,
                 double* weights) {
    const Tables& T = tables(p);
    const double wf = radius * radius;
    for (int j = 0; j <= p; ++j)
        for (int k = 0; k < T.nphi; ++k) {
            const int id = j * T.nphi + k;
            const double v[3] = {T.st[j] * T.cph[k], T.st[j] * T.sph[k], T.ct[j]};
            double o[3];
            qrot(quat, v, o);
            for (int d = 0; d < 3; ++d) {
                if (norms) norms[3 * id + d] = o[d];
                if (coords) coords[3 * id + d] = radius * o[d] + (center ? center[d] : 0.0);
            }
            if (weights) weights[id] = wf * T.wq[j];
        }
}

void orc_sh_g2s(int p, const double* quat, const double* grid3, double* coeff) {
    sh_g2s(p, quat, grid3, reinterpret_cast<cd*>(coeff));
}

void orc_sh_s2g(int p, const double* quat, const double* coeff, double* grid3) {
    const int ng = (p + 1) * (2 * p + 2);
    std::vector<double> g(3 * ng);
    sh_s2g_body(p, reinterpret_cast<const cd*>(coeff), g.data());
    for (int i = 0; i < ng; ++i) qrot(quat, &g[3 * i], grid3 + 3 * i);
}

void orc_sh_self(int p, double radius, const double* quat, const double* coeff, int kind, double* grid3) {
    const int nc = ncoef(p), ng = (p + 1) * (2 * p + 2);
    std::vector<cd> o(3 * nc);
    self_multiply(p, reinterpret_cast<const cd*>(coeff), kind, o.data());
    std::vector<double> g(3 * ng);
    sh_s2g_body(p, o.data(), g.data());
    const double s = kind == 0 ? radius : 1.0;
    for (int i = 0; i < ng; ++i) {
        double v[3];
        qrot(quat, &g[3 * i], v);
        for (int k = 0; k < 3; ++k) grid3[3 * i + k] = s * v[k];
    }
}

void orc_sh_eval_exterior(int p, double radius, const double* quat, const double* coeff, int nt,
                          const double* trg_rel, const double* trg_norm, double* sl_out, double* trac_out) {
    NearSource S;
    near_prepare(p, reinterpret_cast<const cd*>(coeff), S);
    std::vector<double> re(S.nc), im(S.nc);
    for (int i = 0; i < nt; ++i) {
        double xb[3], nb[3] = {0, 0, 1}, u[3], t[3], o[3];
        qinvrot(quat, trg_rel + 3 * i, xb);
        for (int k = 0; k < 3; ++k) xb[k] /= radius;
        if (trg_norm) qinvrot(quat, trg_norm + 3 * i, nb);
        near_eval_point(S, xb, nb, sl_out ? u : nullptr, trac_out ? t : nullptr, re, im);
        if (sl_out) {
            qrot(quat, u, o);
            for (int k = 0; k < 3; ++k) sl_out[3 * i + k] = radius * o[k];
        }
        if (trac_out) {
            qrot(quat, t, o);
            for (int k = 0; k < 3; ++k) trac_out[3 * i + k] = o[k];
        }
    }
}

int orc_near_pairs(int n, const double* centers, const double* radii, int cap, int* trg, int* src) {
    std::vector<int> pt, ps;
    build_pairs(n, centers, radii, pt, ps);
    for (int i = 0; i < (int)pt.size() && i < cap; ++i) {
        trg[i] = pt[i];
        src[i] = ps[i];
    }
    return (int)pt.size();
}

void* orc_create(int n, const double* centers, const double* radii, const double* quats, const int* orders,
                 double viscosity) {
    auto* C = new Ctx;
    C->N = n;
    C->centers.assign(centers, centers + 3 * n);
    C->radii.assign(radii, radii + n);
    C->has_quat = quats != nullptr;
    if (quats) C->quats.assign(quats, quats + 4 * n);
    C->orders.assign(orders, orders + n);
    C->viscosity = viscosity;
    C->gidx.resize(n);
    C->glen.resize(n);
    int off = 0;
    for (int i = 0; i < n; ++i) {
        C->gidx[i] = off;
        C->glen[i] = orc_grid_number(orders[i]);
        off += C->glen[i];
    }
    C->M = off;
    C->coords.resize(3 * off);
    C->norms.resize(3 * off);
    C->weights.resize(off);
    C->sid.resize(off);
    for (int i = 0; i < n; ++i) {
        orc_sh_grid(orders[i], radii[i], C->q(i), &centers[3 * i], &C->coords[3 * C->gidx[i]],
                    &C->norms[3 * C->gidx[i]], &C->weights[C->gidx[i]]);
        for (int j = 0; j < C->glen[i]; ++j) C->sid[C->gidx[i] + j] = i;
    }
    build_pairs(n, centers, radii, C->ptrg, C->psrc);
    return C;
}

void orc_destroy(void* ctx) { delete static_cast<Ctx*>(ctx); }
int orc_num_points(void* ctx) { return static_cast<Ctx*>(ctx)->M; }
int orc_num_pairs(void* ctx) { return (int)static_cast<Ctx*>(ctx)->ptrg.size(); }
void orc_get_pairs(void* ctx, int* trg, int* src) {
    auto* C = static_cast<Ctx*>(ctx);
    std::copy(C->ptrg.begin(), C->ptrg.end(), trg);
    std::copy(C->psrc.begin(), C->psrc.end(), src);
}
void orc_get_grid(void* ctx, double* coords, double* norms, double* weights) {
    auto* C = static_cast<Ctx*>(ctx);
    if (coords) std::copy(C->coords.begin(), C->coords.end(), coords);
    if (norms) std::copy(C->norms.begin(), C->norms.end(), norms);
    if (weights) std::copy(C->weights.begin(), C->weights.end(), weights);
}
void orc_apply_p2p(void* ctx, const double* in, double* out, double cId, double cSL, double cTrac) {
    apply_p2p(*static_cast<Ctx*>(ctx), in, out, cId, cSL, cTrac);
}
void orc_apply_lop(void* ctx, const double* in, double* out, double cLOP) {
    apply_lop(*static_cast<Ctx*>(ctx), in, out, cLOP);
}
void orc_apply(void* ctx, const double* x, double* y, double alpha, double beta) {
    auto* C = static_cast<Ctx*>(ctx);
    std::vector<double> t(3 * C->M);
    apply_A(*C, x, t.data());
    for (int i = 0; i < 3 * C->M; ++i) y[i] = (beta == 0 ? 0.0 : beta * y[i]) + alpha * t[i];
}
void orc_far_traction(void* ctx, const double* in, double* out, double c, int excl_near) {
    far_field(*static_cast<Ctx*>(ctx), in, out, c, true, excl_near != 0);
}
void orc_far_sl(void* ctx, const double* in, double* out, double c, int excl_near) {
    far_field(*static_cast<Ctx*>(ctx), in, out, c, false, excl_near != 0);
}
void orc_near_correction(void* ctx, const double* in, double* out, double c_sl, double c_trac) {
    auto* C = static_cast<Ctx*>(ctx);
    std::vector<std::vector<cd>> coef;
    coeffs_all(*C, in, coef);
    near_terms(*C, coef, in, out, c_sl, c_trac);
}

int orc_solve_mob(void* ctx, const double* force, double* vel, double* density, double tol, int restart, int maxit,
                  int* iters, double* relres) {
    auto* C = static_cast<Ctx*>(ctx);
    const int M = C->M;
    std::vector<double> rho(3 * M), b(3 * M, 0.0), mu(3 * M, 0.0), u(3 * M, 0.0);
    // step 1: rigid density (SphereSTKMobMat.cpp:174-192)
    for (int i = 0; i < C->N; ++i) {
        const double a = C->radii[i];
        const double* F = force + 6 * i;
        const double A[3] = {F[0] / (4 * PI * a * a), F[1] / (4 * PI * a * a), F[2] / (4 * PI * a * a)};
        const double fb = 3.0 / (8 * PI * a * a * a * a);
        const double B[3] = {F[3] * fb, F[4] * fb, F[5] * fb};
        for (int j = 0; j < C->glen[i]; ++j) {
            const int id = C->gidx[i] + j;
            const double* n = &C->norms[3 * id];
            const double r[3] = {a * n[0], a * n[1], a * n[2]};
            rho[3 * id] = A[0] + B[1] * r[2] - B[2] * r[1];
            rho[3 * id + 1] = A[1] + B[2] * r[0] - B[0] * r[2];
            rho[3 * id + 2] = A[2] + B[0] * r[1] - B[1] * r[0];
        }
    }
    // step 2: b = -(I/2 + K) rho
    apply_p2p(*C, rho.data(), b.data(), -0.5, 0, -1.0);
    const double bn = std::sqrt(dot(b, b));
    int it = 0;
    double rr = 0;
    int status = 0;
    if (bn >= 1e-5) status = gmres(*C, b, mu, tol, restart, maxit, &it, &rr);  // SphereSTKMobMat.cpp:216-241
    // step 4: rho + mu, single-layer velocity, rigid averages
    for (int i = 0; i < 3 * M; ++i) rho[i] += mu[i];
    apply_p2p(*C, rho.data(), u.data(), 0, 1.0, 0);
    const double iv = 1.0 / C->viscosity;
    for (int i = 0; i < C->N; ++i) {
        const double a = C->radii[i];
        double V[3] = {0, 0, 0}, W[3] = {0, 0, 0};
        for (int j = 0; j < C->glen[i]; ++j) {
            const int id = C->gidx[i] + j;
            const double w = C->weights[id];
            const double* n = &C->norms[3 * id];
            const double* v = &u[3 * id];
            for (int k = 0; k < 3; ++k) V[k] += w * v[k];
            W[0] += a * w * (n[1] * v[2] - n[2] * v[1]);
            W[1] += a * w * (n[2] * v[0] - n[0] * v[2]);
            W[2] += a * w * (n[0] * v[1] - n[1] * v[0]);
        }
        for (int k = 0; k < 3; ++k) {
            vel[6 * i + k] = V[k] / (4 * PI * a * a) * iv;
            vel[6 * i + 3 + k] = W[k] * 3.0 / (8 * PI * a * a * a * a) * iv;
        }
    }
    if (density) std::copy(rho.begin(), rho.end(), density);
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return status;
}

}  // extern "C"
