// sphere.cu — per-sphere kernels: vector spherical-harmonic transforms, the spectral self
// operators, identity, rigid-body projection L, rigid density and rigid averages.
//
// Reference counterparts:
//   Shexp::calcSpectralCoeff / calcGridValue (Sphere/Shexp.cpp:342-447): forward (G2S) and
//     inverse (S2G) transforms with the layer rotation (invrotGridValue/rotGridValue :449-480);
//   self corrections of applyP2POP (BIE/SphereSTKSHOperator.cpp:306-351 single layer,
//     :375-456 traction principal value 0.5*(KSelf_ext + KSelf_int));
//   identity term (:459-466) and applyLOP (:487-521);
//   rigid density and rigid averages of solveMob (BIE/SphereSTKMobMat.cpp:174-192, 261-285).
//
// One CTA per sphere. The forward transform is a length-(2p+2) DFT per theta ring of the
// spherical components (V_r, V_theta, V_phi) followed by the Legendre contraction over the
// p+1 rings; the self operator is diagonal per degree n in the basis
//   H_n = ((n+1) Y r - grad_s Y)/(2n+1), G_n = n Y r + grad_s Y, X_n = r x grad_s Y
// with multipliers
//   single layer: n/((2n+1)(2n+3)), (n+1)/((2n-1)(2n+1)), 1/(2n+1)   (times the radius)
//   traction PV : 3/(2(2n+1)(2n+3)), -3/(2(2n-1)(2n+1)), -3/(2(2n+1))
// and the inverse transform mirrors the forward one. All stages stay in shared memory.
#include "smob_internal.h"

namespace smob {

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

__device__ __forceinline__ void qrot(const double* q, const double* v, double* o) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double tx = 2 * (y * v[2] - z * v[1]);
    const double ty = 2 * (z * v[0] - x * v[2]);
    const double tz = 2 * (x * v[1] - y * v[0]);
    o[0] = v[0] + w * tx + (y * tz - z * ty);
    o[1] = v[1] + w * ty + (z * tx - x * tz);
    o[2] = v[2] + w * tz + (x * ty - y * tx);
}
__device__ __forceinline__ void qinvrot(const double* q, const double* v, double* o) {
    const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
    qrot(qc, v, o);
}

__device__ __forceinline__ void decode_nm(int idx, int& n, int& m) {
    n = int((sqrtf(8.f * idx + 1.f) - 1.f) * 0.5f);
    while ((n + 1) * (n + 2) / 2 <= idx) ++n;
    while (n * (n + 1) / 2 > idx) --n;
    m = idx - n * (n + 1) / 2;
}

template <typename Real>
__device__ __forceinline__ Real block_sum_to_all(Real v, Real* red) {
    // all threads must call; red holds >= 32 entries
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    Real s = 0;
    const int nw = (blockDim.x + 31) >> 5;
    for (int i = 0; i < nw; ++i) s += red[i];
    return s;
}

struct SphereArgs {
    const double* x;        // grid input (OP, G2S)
    const double* coef_in;  // coefficient input (S2G), double complex
    double* out;            // grid output
    double c_id, c_self, c_lop;
    int self_kind;          // -1 none, 0 single layer, 3 traction PV, 4 block-diagonal preconditioner
    int mode;               // 0 OP, 1 G2S, 2 S2G
    void* coef_out;         // coefficient output (Real complex in OP, double in G2S), may be null
};

template <typename Real>
__global__ void __launch_bounds__(kSphereThreads) k_sphere(DevGeom g, const Real* __restrict__ tab, SphereArgs a) {
    const int s = blockIdx.x;
    if (g.active && !g.active[g.prob[s]]) return;
    const int p = g.order[s];
    const OrderTables T = g.tabs[p];
    const int nt = T.nt, nphi = T.nphi, nc = T.nc, ng = g.glen[s], g0 = g.gidx[s];
    const int P1 = p + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real* vr = reinterpret_cast<Real*>(smem_raw);
    Real* vt = vr + ng;
    Real* vp = vt + ng;
    Real* F = vp + ng;             // [3][nt][P1] complex
    Real* C = F + 6 * nt * P1;     // [3][nc] complex
    __shared__ double red[32];
    const double q[4] = {g.quat[4 * s], g.quat[4 * s + 1], g.quat[4 * s + 2], g.quat[4 * s + 3]};
    const double rad = g.radius[s];
    const Real* ct = tab + T.ring;
    const Real* st = ct + nt;
    const Real* wq = st + nt;
    const Real* Pt = tab + T.leg;
    const Real* dPt = Pt + nt * nc;
    const Real* Pst = dPt + nt * nc;
    const Real* cosm = tab + T.twiddle;
    const Real* sinm = cosm + P1 * nphi;
    const Real* cph = tab + T.cph;
    const Real* sph = cph + nphi;
    const bool want_lop = a.mode == 0 && a.c_lop != 0.0;
    double A[3] = {0, 0, 0}, B[3] = {0, 0, 0};

    if (a.mode != 2) {
        double la[6] = {0, 0, 0, 0, 0, 0};
        for (int i = threadIdx.x; i < ng; i += blockDim.x) {
            const int j = i / nphi, k = i - j * nphi;
            const double v[3] = {a.x[3 * (g0 + i)], a.x[3 * (g0 + i) + 1], a.x[3 * (g0 + i) + 2]};
            if (want_lop) {
                const double w = g.weights[g0 + i];
                const double* n = g.norms + 3 * (g0 + i);
                la[0] += w * v[0];
                la[1] += w * v[1];
                la[2] += w * v[2];
                la[3] += w * rad * (n[1] * v[2] - n[2] * v[1]);
                la[4] += w * rad * (n[2] * v[0] - n[0] * v[2]);
                la[5] += w * rad * (n[0] * v[1] - n[1] * v[0]);
            }
            if (a.self_kind >= 0 || a.mode == 1) {
                double b[3];
                qinvrot(q, v, b);
                const Real cp = cph[k], sp = sph[k], c0 = ct[j], s0 = st[j];
                const Real h = Real(b[0]) * cp + Real(b[1]) * sp;
                vr[i] = h * s0 + Real(b[2]) * c0;
                vt[i] = h * c0 - Real(b[2]) * s0;
                vp[i] = -Real(b[0]) * sp + Real(b[1]) * cp;
            }
        }
        if (want_lop) {
            for (int c = 0; c < 6; ++c) la[c] = block_sum_to_all(la[c], red);
            const double fa = 1.0 / (4 * kPi * rad * rad), fb = 3.0 / (8 * kPi * rad * rad * rad * rad);
            for (int c = 0; c < 3; ++c) {
                A[c] = la[c] * fa;
                B[c] = la[3 + c] * fb;
            }
        }
        if (a.self_kind >= 0 || a.mode == 1) {
            __syncthreads();
            // DFT along phi per ring, m = 0..p
            for (int it = threadIdx.x; it < 3 * nt * P1; it += blockDim.x) {
                const int c = it / (nt * P1), rem = it - c * nt * P1, j = rem / P1, m = rem - j * P1;
                const Real* V = (c == 0 ? vr : (c == 1 ? vt : vp)) + j * nphi;
                const Real* cm = cosm + m * nphi;
                const Real* sm = sinm + m * nphi;
                Real re = 0, im = 0;
                for (int k = 0; k < nphi; ++k) {
                    re += V[k] * cm[k];
                    im -= V[k] * sm[k];
                }
                F[2 * it] = re;
                F[2 * it + 1] = im;
            }
            __syncthreads();
            // Legendre contraction over rings
            for (int idx = threadIdx.x; idx < nc; idx += blockDim.x) {
                int n, m;
                decode_nm(idx, n, m);
                Real rr = 0, ri = 0, gr = 0, gi = 0, xr = 0, xi = 0;
                for (int j = 0; j < nt; ++j) {
                    const Real w = wq[j];
                    const Real P = Pt[j * nc + idx] * w, dP = dPt[j * nc + idx] * w, mPs = Real(m) * Pst[j * nc + idx] * w;
                    const Real* Fr = F + 2 * (j * P1 + m);
                    const Real* Ft = F + 2 * (nt * P1 + j * P1 + m);
                    const Real* Fp = F + 2 * (2 * nt * P1 + j * P1 + m);
                    rr += Fr[0] * P;
                    ri += Fr[1] * P;
                    // (Ft dP - i m Ps Fp)
                    gr += Ft[0] * dP + mPs * Fp[1];
                    gi += Ft[1] * dP - mPs * Fp[0];
                    // (Fp dP + i m Ps Ft)
                    xr += Fp[0] * dP - mPs * Ft[1];
                    xi += Fp[1] * dP + mPs * Ft[0];
                }
                const Real inv = n > 0 ? Real(1) / Real(n * (n + 1)) : Real(0);
                C[2 * idx] = rr;
                C[2 * idx + 1] = ri;
                C[2 * (nc + idx)] = gr * inv;
                C[2 * (nc + idx) + 1] = gi * inv;
                C[2 * (2 * nc + idx)] = xr * inv;
                C[2 * (2 * nc + idx) + 1] = xi * inv;
                if (a.coef_out) {
                    const long long o = 2LL * g.coff[s];
                    if (a.mode == 1) {
                        double* co = static_cast<double*>(a.coef_out) + o;
                        co[2 * idx] = rr;
                        co[2 * idx + 1] = ri;
                        co[2 * (nc + idx)] = gr * inv;
                        co[2 * (nc + idx) + 1] = gi * inv;
                        co[2 * (2 * nc + idx)] = xr * inv;
                        co[2 * (2 * nc + idx) + 1] = xi * inv;
                    } else {
                        Real* co = static_cast<Real*>(a.coef_out) + o;
                        co[2 * idx] = rr;
                        co[2 * idx + 1] = ri;
                        co[2 * (nc + idx)] = gr * inv;
                        co[2 * (nc + idx) + 1] = gi * inv;
                        co[2 * (2 * nc + idx)] = xr * inv;
                        co[2 * (2 * nc + idx) + 1] = xi * inv;
                    }
                }
            }
            if (a.mode == 1) return;
            __syncthreads();
        }
    } else {
        for (int i = threadIdx.x; i < 6 * nc; i += blockDim.x) C[i] = Real(a.coef_in[2LL * g.coff[s] + i]);
        __syncthreads();
    }

    const bool do_inverse = a.mode == 2 || a.self_kind >= 0;
    if (do_inverse) {
        if (a.mode == 0) {
            // self multipliers (in place)
            for (int idx = threadIdx.x; idx < nc; idx += blockDim.x) {
                int n, m;
                decode_nm(idx, n, m);
                const Real dn = Real(n);
                Real lh, lg, lx;
                if (a.self_kind == 0) {
                    lh = dn / ((2 * dn + 1) * (2 * dn + 3));
                    lg = (dn + 1) / ((2 * dn - 1) * (2 * dn + 1));
                    lx = Real(1) / (2 * dn + 1);
                } else if (a.self_kind == 4) {
                    // block-diagonal preconditioner: the inverse of the sphere's own I/2 + K_PV + L,
                    // minus the 2 I that c_id = 2 adds on the grid (that 2 I also inverts the I/2 the
                    // operator applies to the part of a grid field beyond degree p). L is the identity
                    // on the rigid modes (n = 1 G: translations, n = 1 X: rotations), zero elsewhere.
                    const Real dh = Real(0.5) + Real(3) / (2 * (2 * dn + 1) * (2 * dn + 3));
                    const Real dg = n == 1 ? Real(1) : Real(0.5) - Real(3) / (2 * (2 * dn - 1) * (2 * dn + 1));
                    const Real dx = n == 1 ? Real(1) : Real(0.5) - Real(3) / (2 * (2 * dn + 1));
                    lh = Real(1) / dh - 2;
                    lg = Real(1) / dg - 2;
                    lx = Real(1) / dx - 2;
                } else {
                    lh = Real(3) / (2 * (2 * dn + 1) * (2 * dn + 3));
                    lg = Real(-3) / (2 * (2 * dn - 1) * (2 * dn + 1));
                    lx = Real(-3) / (2 * (2 * dn + 1));
                }
                Real* cr = C + 2 * idx;
                Real* cs = C + 2 * (nc + idx);
                Real* cx = C + 2 * (2 * nc + idx);
                for (int c = 0; c < 2; ++c) {
                    const Real h = (cr[c] - dn * cs[c]) * lh;
                    const Real gg = (cr[c] + (dn + 1) * cs[c]) / (2 * dn + 1) * lg;
                    cr[c] = h * ((dn + 1) / (2 * dn + 1)) + dn * gg;
                    cs[c] = n > 0 ? (-h / (2 * dn + 1) + gg) : Real(0);
                    cx[c] = n > 0 ? lx * cx[c] : Real(0);
                }
            }
            __syncthreads();
        }
        // inverse Legendre per (ring, m)
        for (int it = threadIdx.x; it < nt * P1; it += blockDim.x) {
            const int j = it / P1, m = it - j * P1;
            Real r0 = 0, r1 = 0, t0 = 0, t1 = 0, q0 = 0, q1 = 0;
            for (int n = m; n <= p; ++n) {
                const int id = cidx(n, m);
                const Real P = Pt[j * nc + id], dP = dPt[j * nc + id], mPs = Real(m) * Pst[j * nc + id];
                const Real* cr = C + 2 * id;
                const Real* cs = C + 2 * (nc + id);
                const Real* cx = C + 2 * (2 * nc + id);
                r0 += cr[0] * P;
                r1 += cr[1] * P;
                // as dP - i m Ps ax
                t0 += cs[0] * dP + mPs * cx[1];
                t1 += cs[1] * dP - mPs * cx[0];
                // i m Ps as + ax dP
                q0 += -mPs * cs[1] + cx[0] * dP;
                q1 += mPs * cs[0] + cx[1] * dP;
            }
            const Real e = m == 0 ? Real(1) : Real(2);
            Real* Gr = F + 2 * (j * P1 + m);
            Real* Gt = F + 2 * (nt * P1 + j * P1 + m);
            Real* Gp = F + 2 * (2 * nt * P1 + j * P1 + m);
            Gr[0] = e * r0;
            Gr[1] = e * r1;
            Gt[0] = e * t0;
            Gt[1] = e * t1;
            Gp[0] = e * q0;
            Gp[1] = e * q1;
        }
        __syncthreads();
    }

    const double scale = (a.self_kind == 0) ? a.c_self * rad : a.c_self;
    for (int i = threadIdx.x; i < ng; i += blockDim.x) {
        const int j = i / nphi, k = i - j * nphi;
        double o[3] = {0, 0, 0};
        if (do_inverse) {
            Real sr = 0, stt = 0, sp = 0;
            for (int m = 0; m <= p; ++m) {
                const Real c0 = cosm[m * nphi + k], s0 = sinm[m * nphi + k];
                const Real* Gr = F + 2 * (j * P1 + m);
                const Real* Gt = F + 2 * (nt * P1 + j * P1 + m);
                const Real* Gp = F + 2 * (2 * nt * P1 + j * P1 + m);
                sr += Gr[0] * c0 - Gr[1] * s0;
                stt += Gt[0] * c0 - Gt[1] * s0;
                sp += Gp[0] * c0 - Gp[1] * s0;
            }
            const Real cp = cph[k], spp = sph[k], c0 = ct[j], s0 = st[j];
            const double b[3] = {double(sr * s0 * cp + stt * c0 * cp - sp * spp),
                                 double(sr * s0 * spp + stt * c0 * spp + sp * cp), double(sr * c0 - stt * s0)};
            qrot(q, b, o);
        }
        double* dst = a.out + 3 * (g0 + i);
        if (a.mode == 2) {
            dst[0] = o[0];
            dst[1] = o[1];
            dst[2] = o[2];
            continue;
        }
        double add[3] = {0, 0, 0};
        if (a.self_kind >= 0)
            for (int c = 0; c < 3; ++c) add[c] += scale * o[c];
        if (a.c_id != 0.0)
            for (int c = 0; c < 3; ++c) add[c] += a.c_id * a.x[3 * (g0 + i) + c];
        if (want_lop) {
            const double* n = g.norms + 3 * (g0 + i);
            const double r[3] = {rad * n[0], rad * n[1], rad * n[2]};
            add[0] += a.c_lop * (A[0] + B[1] * r[2] - B[2] * r[1]);
            add[1] += a.c_lop * (A[1] + B[2] * r[0] - B[0] * r[2]);
            add[2] += a.c_lop * (A[2] + B[0] * r[1] - B[1] * r[0]);
        }
        dst[0] += add[0];
        dst[1] += add[1];
        dst[2] += add[2];
    }
}

template <typename Real>
size_t sphere_smem(int pmax) {
    const int ng = (pmax + 1) * (2 * pmax + 2), nt = pmax + 1, P1 = pmax + 1, nc = ncoef(pmax);
    return size_t(3 * ng + 6 * nt * P1 + 6 * nc) * sizeof(Real);
}

template <typename Real>
const Real* table_of(const DevGeom& g);
template <>
const float* table_of<float>(const DevGeom& g) { return g.tab_f; }
template <>
const double* table_of<double>(const DevGeom& g) { return g.tab_d; }

template <typename Real>
int launch_sphere(const DevGeom& g, SphereArgs a, cudaStream_t st) {
    k_sphere<Real><<<g.N, kSphereThreads, sphere_smem<Real>(g.pmax), st>>>(g, table_of<Real>(g), a);
    return 1;
}

__global__ void k_rigid_density(DevGeom g, const double* __restrict__ f6, double* __restrict__ rho) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.M) return;
    const int s = g.sid[i];
    if (g.active && !g.active[g.prob[s]]) return;
    const double a = g.radius[s];
    const double* F = f6 + 6 * s;
    const double fa = 1.0 / (4 * kPi * a * a), fb = 3.0 / (8 * kPi * a * a * a * a);
    const double* n = g.norms + 3 * i;
    const double r[3] = {a * n[0], a * n[1], a * n[2]};
    const double B[3] = {F[3] * fb, F[4] * fb, F[5] * fb};
    rho[3 * i] = F[0] * fa + B[1] * r[2] - B[2] * r[1];
    rho[3 * i + 1] = F[1] * fa + B[2] * r[0] - B[0] * r[2];
    rho[3 * i + 2] = F[2] * fa + B[0] * r[1] - B[1] * r[0];
}

// Grid points, normals and the far-field copies of every point from the spheres' current centres and
// orientations (Shexp::getGridWithPole without the poles, Sphere/Shexp.cpp:206-271). The one builder
// of the grid, at context creation and after every geometry update, so an updated context equals a
// newly created one bit for bit; explicit round-to-nearest operations keep the result independent
// of the compiler's FMA contraction.
__device__ __forceinline__ void qrot_rn(const double* q, const double* v, double* o) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double tx = __dmul_rn(2.0, __dsub_rn(__dmul_rn(y, v[2]), __dmul_rn(z, v[1])));
    const double ty = __dmul_rn(2.0, __dsub_rn(__dmul_rn(z, v[0]), __dmul_rn(x, v[2])));
    const double tz = __dmul_rn(2.0, __dsub_rn(__dmul_rn(x, v[1]), __dmul_rn(y, v[0])));
    o[0] = __dadd_rn(__dadd_rn(v[0], __dmul_rn(w, tx)), __dsub_rn(__dmul_rn(y, tz), __dmul_rn(z, ty)));
    o[1] = __dadd_rn(__dadd_rn(v[1], __dmul_rn(w, ty)), __dsub_rn(__dmul_rn(z, tx), __dmul_rn(x, tz)));
    o[2] = __dadd_rn(__dadd_rn(v[2], __dmul_rn(w, tz)), __dsub_rn(__dmul_rn(x, ty), __dmul_rn(y, tx)));
}

__global__ void k_regrid(DevGeom g, const double* __restrict__ org, double* __restrict__ coords,
                         double* __restrict__ norms, float4* __restrict__ pos32, float4* __restrict__ nrm32,
                         float4* __restrict__ pos32lo, float4* __restrict__ nrm32lo, double4_32a* __restrict__ pos64,
                         double4_32a* __restrict__ nrm64) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.M) return;
    const int s = g.sid[i];
    const OrderTables T = g.tabs[g.order[s]];
    const int l = i - g.gidx[s], j = l / T.nphi, k = l - j * T.nphi;
    const double ct = g.tab_d[T.ring + j], st = g.tab_d[T.ring + T.nt + j];
    const double cp = g.tab_d[T.cph + k], sp = g.tab_d[T.cph + T.nphi + k];
    const double v[3] = {__dmul_rn(st, cp), __dmul_rn(st, sp), ct};
    double n[3];
    qrot_rn(g.quat + 4 * s, v, n);
    const double a = g.radius[s];
    const double* o = org + 3 * g.prob[s];
    double x[3], r[3];
    for (int d = 0; d < 3; ++d) {
        x[d] = __dadd_rn(__dmul_rn(a, n[d]), g.center[3 * s + d]);
        r[d] = __dsub_rn(x[d], o[d]);
        coords[3 * i + d] = x[d];
        norms[3 * i + d] = n[d];
    }
    const float4 p = make_float4(float(r[0]), float(r[1]), float(r[2]), __int_as_float(s));
    const float4 q = make_float4(float(n[0]), float(n[1]), float(n[2]), 0.f);
    pos32[i] = p;
    nrm32[i] = q;
    pos32lo[i] = make_float4(float(__dsub_rn(r[0], double(p.x))), float(__dsub_rn(r[1], double(p.y))),
                             float(__dsub_rn(r[2], double(p.z))), 0.f);
    nrm32lo[i] = make_float4(float(__dsub_rn(n[0], double(q.x))), float(__dsub_rn(n[1], double(q.y))),
                             float(__dsub_rn(n[2], double(q.z))), 0.f);
    pos64[i] = make_double4_32a(r[0], r[1], r[2], 0.0);
    nrm64[i] = make_double4_32a(n[0], n[1], n[2], 0.0);
}

// coarse points of one (sphere, level) entry per CTA: the order-pe unit nodes placed like the sphere's
// own grid (k_regrid), relative to the problem origin in FP32 (and the low parts when asked)
__global__ void k_coarse_grid(DevGeom g, CoarseSet cs, const double* __restrict__ org, float4* __restrict__ cpos32,
                              float4* __restrict__ cpos32lo, float4* __restrict__ cnrm32, float4* __restrict__ cnrm32lo) {
    const int2 e = cs.cent[blockIdx.x];
    const int s = e.x;
    const int4 L = cs.clev[s * kCoarseLevels + e.y];
    const double* nodes = g.cnode + 3LL * g.cnode_off[L.x];
    const double a = g.radius[s];
    const double* o = org + 3 * g.prob[s];
    for (int k = threadIdx.x; k < L.z; k += blockDim.x) {
        double n[3], r[3];
        qrot_rn(g.quat + 4 * s, nodes + 3 * k, n);
        for (int d = 0; d < 3; ++d) r[d] = __dsub_rn(__dadd_rn(__dmul_rn(a, n[d]), g.center[3 * s + d]), o[d]);
        const float4 p = make_float4(float(r[0]), float(r[1]), float(r[2]), __int_as_float(s));
        cpos32[L.y + k] = p;
        if (cpos32lo)
            cpos32lo[L.y + k] = make_float4(float(__dsub_rn(r[0], double(p.x))), float(__dsub_rn(r[1], double(p.y))),
                                            float(__dsub_rn(r[2], double(p.z))), 0.f);
        if (cnrm32) {
            const float4 q = make_float4(float(n[0]), float(n[1]), float(n[2]), __int_as_float(e.y));
            cnrm32[L.y + k] = q;
            if (cnrm32lo)
                cnrm32lo[L.y + k] = make_float4(float(__dsub_rn(n[0], double(q.x))), float(__dsub_rn(n[1], double(q.y))),
                                                float(__dsub_rn(n[2], double(q.z))), 0.f);
        }
    }
}

__global__ void k_rigid_average(DevGeom g, const double* __restrict__ u, double inv_visc, double* __restrict__ vel) {
    const int s = blockIdx.x;
    if (g.active && !g.active[g.prob[s]]) return;
    __shared__ double red[32];
    const int g0 = g.gidx[s], ng = g.glen[s];
    const double a = g.radius[s];
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < ng; i += blockDim.x) {
        const double w = g.weights[g0 + i];
        const double* v = u + 3 * (g0 + i);
        const double* n = g.norms + 3 * (g0 + i);
        acc[0] += w * v[0];
        acc[1] += w * v[1];
        acc[2] += w * v[2];
        acc[3] += a * w * (n[1] * v[2] - n[2] * v[1]);
        acc[4] += a * w * (n[2] * v[0] - n[0] * v[2]);
        acc[5] += a * w * (n[0] * v[1] - n[1] * v[0]);
    }
    for (int c = 0; c < 6; ++c) acc[c] = block_sum_to_all(acc[c], red);
    if (threadIdx.x == 0) {
        const double fa = 1.0 / (4 * kPi * a * a), fb = 3.0 / (8 * kPi * a * a * a * a);
        for (int c = 0; c < 3; ++c) {
            vel[6 * s + c] = acc[c] * fa * inv_visc;
            vel[6 * s + 3 + c] = acc[3 + c] * fb * inv_visc;
        }
    }
}

}  // namespace

void configure_sphere_kernels() {
    cudaFuncSetAttribute(k_sphere<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(sphere_smem<float>(kMaxOrder)));
    cudaFuncSetAttribute(k_sphere<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(sphere_smem<double>(kMaxOrder)));
}

int launch_sphere_op(const DevGeom& g, const double* x, double* out, double c_id, double c_self, int self_kind,
                     double c_lop, void* coef, bool fp32, cudaStream_t st) {
    SphereArgs a{x, nullptr, out, c_id, c_self, c_lop, self_kind, 0, coef};
    return fp32 ? launch_sphere<float>(g, a, st) : launch_sphere<double>(g, a, st);
}

int launch_sh_g2s(const DevGeom& g, const double* grid, double* coef, cudaStream_t st) {
    SphereArgs a{grid, nullptr, nullptr, 0, 0, 0, -1, 1, coef};
    return launch_sphere<double>(g, a, st);
}

int launch_sh_s2g(const DevGeom& g, const double* coef, double* grid, cudaStream_t st) {
    SphereArgs a{nullptr, coef, grid, 0, 0, 0, -1, 2, nullptr};
    return launch_sphere<double>(g, a, st);
}

int launch_regrid(const DevGeom& g, const double* org, cudaStream_t st) {
    k_regrid<<<(g.M + 255) / 256, 256, 0, st>>>(g, org, const_cast<double*>(g.coords), const_cast<double*>(g.norms),
                                                const_cast<float4*>(g.pos32), const_cast<float4*>(g.nrm32),
                                                const_cast<float4*>(g.pos32lo), const_cast<float4*>(g.nrm32lo),
                                                const_cast<double4_32a*>(g.pos64), const_cast<double4_32a*>(g.nrm64));
    return 1;
}

int launch_coarse_grid(const DevGeom& g, const CoarseSet& cs, const double* org, float4* cpos32, float4* cpos32lo,
                       float4* cnrm32, float4* cnrm32lo, cudaStream_t st) {
    if (cs.ncent <= 0) return 0;
    k_coarse_grid<<<cs.ncent, 128, 0, st>>>(g, cs, org, cpos32, cpos32lo, cnrm32, cnrm32lo);
    return 1;
}

int launch_rigid_density(const DevGeom& g, const double* force6n, double* rho, cudaStream_t st) {
    k_rigid_density<<<(g.M + 255) / 256, 256, 0, st>>>(g, force6n, rho);
    return 1;
}

int launch_rigid_average(const DevGeom& g, const double* u, double inv_visc, double* vel6n, cudaStream_t st) {
    k_rigid_average<<<g.N, 256, 0, st>>>(g, u, inv_visc, vel6n);
    return 1;
}

}  // namespace smob
