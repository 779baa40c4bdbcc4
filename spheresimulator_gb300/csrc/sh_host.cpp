// sh_host.cpp — host-side spectral precompute (see sh_host.h).
//
// Conventions (the same as the device kernels):
//  * grid of order p: rings j = 0..p at the Gauss-Legendre nodes ordered north to south
//    (cos theta descending, Sphere/Shexp.cpp:226-245), phi_k = 2 pi k/(2p+2);
//  * Ybar_n^m = orthonormal associated Legendre function times e^{i m phi}, no Condon-Shortley phase;
//  * density coefficients: vector spherical harmonics Y r, grad_s Y, r x grad_s Y of degree <= p;
//  * exterior Laplace single layer of a scalar density g on the unit sphere:
//      L[g](x) = Re sum_{n,m>=0} eps_m (-1)^n sqrt(4pi/(2n+1)) g_nm Th_n^m(x),
//    Th_n^m = d_+^m d_z^(n-m) (1/r) / sqrt((n-m)!(n+m)!), so d/dx_i are index shifts;
//  * Stokes single layer and stress from four Laplace potentials (Cartesian density components
//    L_x, L_y, L_z and L_r = L[y.f]):
//      8 pi u_i = L_i - x_j d_i L_j + d_i L_r,   4 pi sigma_ik = delta_ik div L - x_j d_i d_k L_j + d_i d_k L_r.
// The near map is built column by column by running that linear chain on unit coefficients:
// synthesis of the vector field on the order-(p+1) grid, exact scalar analysis of its Cartesian
// components to degree p+1, scaling, and the derivative index shifts.
#include "sh_host.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <map>
#include <memory>
#include <mutex>

#include "smob_internal.h"

namespace smob {
namespace {

using cd = std::complex<double>;
constexpr double PI = 3.14159265358979323846264338327950288;

void legendre_ring(int p, double t, double s, double* P, double* dP, double* Ps) {
    std::vector<double> pp(ncoef(p), 0.0);
    pp[0] = std::sqrt(1.0 / (4 * PI));
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
            const double c = n > 0 ? std::sqrt((double(n) * n - double(m) * m) * (2.0 * n + 1) / (2.0 * n - 1)) : 0.0;
            P[cidx(n, m)] = pp[cidx(n, m)];
            dP[cidx(n, m)] = (n * t * pp[cidx(n, m)] - c * prev) / s;  // d/dtheta (rings never touch the poles)
            Ps[cidx(n, m)] = pp[cidx(n, m)] / s;
        }
}

// synthesis of VSH coefficients of degree <= pc on the grid of table T (body frame, Cartesian output)
void synth(const HostOrderTables& T, int pc, const cd* c, double* g) {
    const int ncc = ncoef(pc);
    std::vector<cd> Gr(pc + 1), Gt(pc + 1), Gp(pc + 1);
    for (int j = 0; j < T.nt; ++j) {
        const double* P = &T.P[j * T.nc];
        const double* dP = &T.dP[j * T.nc];
        const double* Ps = &T.Ps[j * T.nc];
        for (int m = 0; m <= pc; ++m) {
            cd r(0, 0), t(0, 0), q(0, 0);
            for (int n = m; n <= pc; ++n) {
                const int id = cidx(n, m);
                const cd im(0, m * Ps[id]);
                r += c[id] * P[id];
                t += c[ncc + id] * dP[id] - im * c[2 * ncc + id];
                q += im * c[ncc + id] + c[2 * ncc + id] * dP[id];
            }
            const double e = m == 0 ? 1.0 : 2.0;
            Gr[m] = e * r;
            Gt[m] = e * t;
            Gp[m] = e * q;
        }
        for (int k = 0; k < T.nphi; ++k) {
            double vr = 0, vt = 0, vp = 0;
            for (int m = 0; m <= pc; ++m) {
                const double c0 = T.cosmk[m * T.nphi + k], s0 = T.sinmk[m * T.nphi + k];
                vr += Gr[m].real() * c0 - Gr[m].imag() * s0;
                vt += Gt[m].real() * c0 - Gt[m].imag() * s0;
                vp += Gp[m].real() * c0 - Gp[m].imag() * s0;
            }
            const double cp = T.cph[k], sp = T.sph[k], ct = T.ct[j], st = T.st[j];
            double* v = g + 3 * (j * T.nphi + k);
            v[0] = vr * st * cp + vt * ct * cp - vp * sp;
            v[1] = vr * st * sp + vt * ct * sp + vp * cp;
            v[2] = vr * ct - vt * st;
        }
    }
}

}  // namespace

// the VSH expansion of degree <= p at one body-frame direction (theta, phi), Cartesian body-frame
// output; the same basis and sums as synth (0 < theta < pi)
void vsh_eval_point(int p, const std::complex<double>* c, double theta, double phi, double* out) {
    const int nc = ncoef(p);
    std::vector<double> P(nc), dP(nc), Ps(nc);
    const double t = std::cos(theta), s = std::sin(theta);
    legendre_ring(p, t, s, P.data(), dP.data(), Ps.data());
    double vr = 0, vt = 0, vp = 0;
    for (int m = 0; m <= p; ++m) {
        cd r(0, 0), th(0, 0), q(0, 0);
        for (int n = m; n <= p; ++n) {
            const int id = cidx(n, m);
            const cd im(0, m * Ps[id]);
            r += c[id] * P[id];
            th += c[nc + id] * dP[id] - im * c[2 * nc + id];
            q += im * c[nc + id] + c[2 * nc + id] * dP[id];
        }
        const double e = m == 0 ? 1.0 : 2.0, c0 = std::cos(m * phi), s0 = std::sin(m * phi);
        vr += e * (r.real() * c0 - r.imag() * s0);
        vt += e * (th.real() * c0 - th.imag() * s0);
        vp += e * (q.real() * c0 - q.imag() * s0);
    }
    const double cp = std::cos(phi), sp = std::sin(phi);
    out[0] = vr * s * cp + vt * t * cp - vp * sp;
    out[1] = vr * s * sp + vt * t * sp + vp * cp;
    out[2] = vr * t - vt * s;
}

namespace {

void scalar_analysis(const HostOrderTables& T, const double* f, int stride, cd* out) {
    const int pd = T.p;
    std::fill(out, out + ncoef(pd), cd(0, 0));
    std::vector<cd> F(pd + 1);
    for (int j = 0; j < T.nt; ++j) {
        std::fill(F.begin(), F.end(), cd(0, 0));
        for (int k = 0; k < T.nphi; ++k) {
            const double v = f[stride * (j * T.nphi + k)];
            for (int m = 0; m <= pd; ++m) F[m] += v * cd(T.cosmk[m * T.nphi + k], -T.sinmk[m * T.nphi + k]);
        }
        for (int n = 0; n <= pd; ++n)
            for (int m = 0; m <= n; ++m) out[cidx(n, m)] += T.wq[j] * F[m] * T.P[j * T.nc + cidx(n, m)];
    }
}

// derivative of F = Re sum c Th (degree <= N) along axis -> degree N+1 (out overwritten, size ncoef(N+1))
void dshift(const cd* c, int N, int axis, cd* out) {
    std::fill(out, out + ncoef(N + 1), cd(0, 0));
    const cd I(0, 1);
    for (int n = 0; n <= N; ++n)
        for (int m = 0; m <= n; ++m) {
            const cd cc = c[cidx(n, m)];
            if (cc == cd(0, 0)) continue;
            const double ap = std::sqrt(double(n + m + 1) * (n + m + 2));
            const double am = std::sqrt(double(n - m + 1) * (n - m + 2));
            if (axis == 2) {
                out[cidx(n + 1, m)] += cc * std::sqrt(double(n + 1) * (n + 1) - double(m) * m);
            } else if (axis == 0) {
                if (m == 0) {
                    out[cidx(n + 1, 1)] += ap * cc.real();
                } else {
                    out[cidx(n + 1, m + 1)] += 0.5 * ap * cc;
                    out[cidx(n + 1, m - 1)] -= 0.5 * am * cc;
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

inline int sym(int i, int k) {
    if (i == k) return i;
    if (i > k) std::swap(i, k);
    return (i == 0) ? (k == 1 ? 3 : 4) : 5;
}

// the linear chain for one coefficient vector: returns sets at degree p+3, [set][idx]
void near_chain(int p, const cd* coeff, bool trac, std::vector<cd>& sets) {
    const int q = p + 1, Nd = p + 3, nc = ncoef(Nd);
    const int ns = trac ? kNearSetsTrac : kNearSetsSL;
    sets.assign(size_t(ns) * nc, cd(0, 0));
    const HostOrderTables& Tq = host_tables(q);
    std::vector<double> g(3 * Tq.nt * Tq.nphi);
    synth(Tq, p, coeff, g.data());
    std::vector<std::vector<cd>> L(4, std::vector<cd>(ncoef(q), cd(0, 0)));
    for (int k = 0; k < 3; ++k) scalar_analysis(Tq, g.data() + k, 3, L[k].data());
    for (int n = 0; n <= p; ++n)
        for (int m = 0; m <= n; ++m) L[3][cidx(n, m)] = coeff[cidx(n, m)];
    for (int k = 0; k < 4; ++k)
        for (int n = 0; n <= q; ++n)
            for (int m = 0; m <= n; ++m)
                L[k][cidx(n, m)] *= (m == 0 ? 1.0 : 2.0) * ((n & 1) ? -1.0 : 1.0) * std::sqrt(4 * PI / (2.0 * n + 1));
    std::vector<cd> t1(ncoef(Nd + 1)), t2(ncoef(Nd + 2));
    auto put = [&](int s, const cd* c, int N) {
        for (int n = 0; n <= std::min(N, Nd); ++n)
            for (int m = 0; m <= n; ++m) sets[size_t(s) * nc + cidx(n, m)] += c[cidx(n, m)];
    };
    if (trac) {
        // 0: div L; 1 + 6j + sym: d_i d_k L_j (j = 0..2); 19 + sym: d_i d_k L_r
        for (int j = 0; j < 4; ++j)
            for (int i = 0; i < 3; ++i) {
                dshift(L[j].data(), q, i, t1.data());
                if (j < 3 && i == j) put(0, t1.data(), q + 1);
                for (int k = i; k < 3; ++k) {
                    dshift(t1.data(), q + 1, k, t2.data());
                    put(j < 3 ? 1 + 6 * j + sym(i, k) : 19 + sym(i, k), t2.data(), q + 2);
                }
            }
    } else {
        // 0..2: L_j; 3 + 3j + i: d_i L_j; 12 + i: d_i L_r
        for (int j = 0; j < 3; ++j) put(j, L[j].data(), q);
        for (int j = 0; j < 4; ++j)
            for (int i = 0; i < 3; ++i) {
                dshift(L[j].data(), q, i, t1.data());
                put(j < 3 ? 3 + 3 * j + i : 12 + i, t1.data(), q + 1);
            }
    }
}

}  // namespace

void gauss_legendre_nodes(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(PI * (i + 0.75) / (n + 0.5)), dp = 0;
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
        double p0 = 1, p1 = 0;
        for (int k = 1; k <= n; ++k) {
            const double p2 = p1;
            p1 = p0;
            p0 = ((2 * k - 1) * z * p1 - (k - 1) * p2) / k;
        }
        dp = n * (z * p0 - p1) / (z * z - 1);
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1 - z * z) * dp * dp);
    }
}

const HostOrderTables& host_tables(int p) {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<HostOrderTables>> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(p);
    if (it != cache.end()) return *it->second;
    auto T = std::make_unique<HostOrderTables>();
    T->p = p;
    T->nt = p + 1;
    T->nphi = 2 * p + 2;
    T->nc = ncoef(p);
    std::vector<double> x, w;
    gauss_legendre_nodes(p + 1, x, w);
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
        T->cph[k] = std::cos(2 * PI * k / T->nphi);
        T->sph[k] = std::sin(2 * PI * k / T->nphi);
    }
    T->cosmk.resize((p + 1) * T->nphi);
    T->sinmk.resize((p + 1) * T->nphi);
    for (int m = 0; m <= p; ++m)
        for (int k = 0; k < T->nphi; ++k) {
            const long mk = (long(m) * k) % T->nphi;
            T->cosmk[m * T->nphi + k] = std::cos(2 * PI * mk / T->nphi);
            T->sinmk[m * T->nphi + k] = std::sin(2 * PI * mk / T->nphi);
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

const SparseMap& near_map(int p, bool trac) {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<SparseMap>> cache;
    const int key = 2 * p + (trac ? 1 : 0);
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return *it->second;
    }
    host_tables(p + 1);  // populate before the parallel section
    const int ncp = ncoef(p), ncols = 6 * ncp, Nd = p + 3, ncd = ncoef(Nd);
    const int ns = trac ? kNearSetsTrac : kNearSetsSL;
    const int rows = 2 * ns * ncd;
    // column-wise dense results, then transpose to CSR
    std::vector<std::vector<std::pair<int, double>>> colent(ncols);
#pragma omp parallel for schedule(dynamic)
    for (int c = 0; c < ncols; ++c) {
        std::vector<cd> coeff(3 * ncp, cd(0, 0)), sets;
        const int reim = c & 1, lin = c >> 1;
        coeff[lin] = reim ? cd(0, 1) : cd(1, 0);
        near_chain(p, coeff.data(), trac, sets);
        double mx = 0;
        for (const cd& v : sets) mx = std::max(mx, std::max(std::fabs(v.real()), std::fabs(v.imag())));
        const double cut = 1e-15 * mx;
        for (int s = 0; s < ns; ++s)
            for (int id = 0; id < ncd; ++id) {
                const cd v = sets[size_t(s) * ncd + id];
                const int r0 = (id * ns + s) * 2;
                if (std::fabs(v.real()) > cut) colent[c].push_back({r0, v.real()});
                if (std::fabs(v.imag()) > cut) colent[c].push_back({r0 + 1, v.imag()});
            }
    }
    auto M = std::make_unique<SparseMap>();
    M->rows = rows;
    M->cols = ncols;
    M->nsets = ns;
    M->rowptr.assign(rows + 1, 0);
    for (int c = 0; c < ncols; ++c)
        for (auto& e : colent[c]) M->rowptr[e.first + 1]++;
    for (int r = 0; r < rows; ++r) M->rowptr[r + 1] += M->rowptr[r];
    M->col.resize(M->rowptr[rows]);
    M->val.resize(M->rowptr[rows]);
    std::vector<int> fill(M->rowptr.begin(), M->rowptr.end() - 1);
    for (int c = 0; c < ncols; ++c)
        for (auto& e : colent[c]) {
            M->col[fill[e.first]] = c;
            M->val[fill[e.first]] = e.second;
            fill[e.first]++;
        }
    std::lock_guard<std::mutex> lk(mu);
    // another thread (e.g. a second server worker) may have built the same map meanwhile: keep the
    // first one, whose address earlier callers already hold
    auto it = cache.find(key);
    if (it != cache.end()) return *it->second;
    auto& ref = *M;
    cache[key] = std::move(M);
    return ref;
}

void unit_nodes(int p, std::vector<double>& xyz) {
    const HostOrderTables& T = host_tables(p);
    xyz.resize(3 * size_t(T.nt) * T.nphi);
    for (int j = 0; j < T.nt; ++j)
        for (int k = 0; k < T.nphi; ++k) {
            double* v = &xyz[3 * (size_t(j) * T.nphi + k)];
            v[0] = T.st[j] * T.cph[k];
            v[1] = T.st[j] * T.sph[k];
            v[2] = T.ct[j];
        }
}

// Equivalent sources on the order-pe grid of the same sphere (FP64 map; coarse_map is its FP32 copy): f_e[k] = W_pe[k] sum_j K(k, j) f[j],
// K(k, j) = sum_{n <= pe} (2n+1)/(4 pi) P_n(nu_k . nu_j) (the addition theorem: the reproducing kernel
// of the harmonics of degree <= pe). f are weighted grid sources (w_j x_j), so with the order-p
// quadrature exact to degree 2p+1 this is the order-p projection of x onto degree <= pe, sampled at
// the coarse nodes and weighted with the coarse quadrature.
const std::vector<double>& coarse_map_d(int p, int pe) {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<std::vector<double>>> cache;
    const int key = p * 64 + pe;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return *it->second;
    }
    const HostOrderTables& Te = host_tables(pe);
    std::vector<double> nf, nc;
    unit_nodes(p, nf);
    unit_nodes(pe, nc);
    const int ng = int(nf.size() / 3), ne = int(nc.size() / 3);
    auto M = std::make_unique<std::vector<double>>(size_t(ng) * ne);
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ng; ++j)
        for (int k = 0; k < ne; ++k) {
            const double x = std::max(-1.0, std::min(1.0, nf[3 * j] * nc[3 * k] + nf[3 * j + 1] * nc[3 * k + 1] +
                                                              nf[3 * j + 2] * nc[3 * k + 2]));
            // Legendre recurrence P_{n+1} = ((2n+1) x P_n - n P_{n-1}) / (n+1)
            double p0 = 1.0, p1 = x, sum = 1.0 + 3.0 * x;
            if (pe == 0) sum = 1.0;
            for (int n = 1; n < pe; ++n) {
                const double p2 = ((2.0 * n + 1) * x * p1 - n * p0) / (n + 1);
                p0 = p1;
                p1 = p2;
                sum += (2.0 * (n + 1) + 1) * p2;
            }
            (*M)[size_t(j) * ne + k] = Te.wq[k / Te.nphi] * sum / (4 * PI);
        }
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return *it->second;
    auto& ref = *M;
    cache[key] = std::move(M);
    return ref;
}

const std::vector<float>& coarse_map(int p, int pe) {
    static std::mutex mu;
    static std::map<int, std::unique_ptr<std::vector<float>>> cache;
    const int key = p * 64 + pe;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return *it->second;
    }
    const std::vector<double>& d = coarse_map_d(p, pe);
    auto M = std::make_unique<std::vector<float>>(d.begin(), d.end());
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return *it->second;
    auto& ref = *M;
    cache[key] = std::move(M);
    return ref;
}

void theta_recurrence(int nmax, std::vector<double>& c1, std::vector<double>& c2, std::vector<double>& diag) {
    c1.assign(ncoef(nmax), 0.0);
    c2.assign(ncoef(nmax), 0.0);
    diag.assign(nmax + 1, 0.0);
    for (int m = 1; m <= nmax; ++m) diag[m] = std::sqrt((2.0 * m - 1) / (2.0 * m));
    for (int n = 0; n <= nmax; ++n)
        for (int m = 0; m <= n; ++m) {
            const double d = double(n + 1) * (n + 1) - double(m) * m;
            c1[cidx(n, m)] = (2.0 * n + 1) / std::sqrt(d);
            c2[cidx(n, m)] = std::sqrt((double(n) * n - double(m) * m) / d);
        }
}

}  // namespace smob
