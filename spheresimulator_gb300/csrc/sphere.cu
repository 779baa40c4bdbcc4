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
#include "tc_sm100.h"

namespace smob {

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

template <typename T>
__device__ __forceinline__ void qrot(const T* q, const T* v, T* o) {
    const T w = q[0], x = q[1], y = q[2], z = q[3];
    const T tx = 2 * (y * v[2] - z * v[1]);
    const T ty = 2 * (z * v[0] - x * v[2]);
    const T tz = 2 * (x * v[1] - y * v[0]);
    o[0] = v[0] + w * tx + (y * tz - z * ty);
    o[1] = v[1] + w * ty + (z * tx - x * tz);
    o[2] = v[2] + w * tz + (x * ty - y * tx);
}
template <typename T>
__device__ __forceinline__ void qinvrot(const T* q, const T* v, T* o) {
    const T qc[4] = {q[0], -q[1], -q[2], -q[3]};
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
    int mode;               // 0 OP, 1 G2S, 2 S2G; the tensor-core operator (FP32): 3 its first stage (rotate,
                            // DFT along phi -> fg, rigid-mode sums -> lop), 4 its last stage (fg holds the
                            // inverse-Legendre values: inverse DFT, rotate back, self, identity and L terms)
    void* coef_out;         // coefficient output (Real complex in OP, double in G2S), may be null
    float* fg;              // modes 3 and 4: per sphere [3][nt][p+1] complex at fg_stride floats per sphere
    long long fg_stride;
    double* lop;            // modes 3 and 4: per sphere the rigid-mode vectors A, B of L (6 doubles)
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
    // rotations and the rigid-mode (L) sums in Real: FP32 in the FP32 operator (the FP64 pipe of this GPU
    // is 1/58 of the FP32 one), FP64 in the FP64 operator
    const Real q[4] = {Real(g.quat[4 * s]), Real(g.quat[4 * s + 1]), Real(g.quat[4 * s + 2]), Real(g.quat[4 * s + 3])};
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
    const bool want_lop = (a.mode == 0 || a.mode == 3 || a.mode == 4) && a.c_lop != 0.0;
    double A[3] = {0, 0, 0}, B[3] = {0, 0, 0};

    if (a.mode != 2 && a.mode != 4) {
        Real la[6] = {0, 0, 0, 0, 0, 0};
        const Real rr = Real(rad);
        for (int i = threadIdx.x; i < ng; i += blockDim.x) {
            const int j = i / nphi, k = i - j * nphi;
            const Real v[3] = {Real(a.x[3 * (g0 + i)]), Real(a.x[3 * (g0 + i) + 1]), Real(a.x[3 * (g0 + i) + 2])};
            if (want_lop) {
                const Real w = Real(g.weights[g0 + i]);
                const Real n[3] = {Real(g.norms[3 * (g0 + i)]), Real(g.norms[3 * (g0 + i) + 1]),
                                   Real(g.norms[3 * (g0 + i) + 2])};
                la[0] += w * v[0];
                la[1] += w * v[1];
                la[2] += w * v[2];
                la[3] += w * rr * (n[1] * v[2] - n[2] * v[1]);
                la[4] += w * rr * (n[2] * v[0] - n[0] * v[2]);
                la[5] += w * rr * (n[0] * v[1] - n[1] * v[0]);
            }
            if (a.self_kind >= 0 || a.mode == 1) {
                Real b[3];
                qinvrot(q, v, b);
                const Real cp = cph[k], sp = sph[k], c0 = ct[j], s0 = st[j];
                const Real h = b[0] * cp + b[1] * sp;
                vr[i] = h * s0 + b[2] * c0;
                vt[i] = h * c0 - b[2] * s0;
                vp[i] = -b[0] * sp + b[1] * cp;
            }
        }
        if (want_lop) {
            for (int c = 0; c < 6; ++c) la[c] = block_sum_to_all(la[c], reinterpret_cast<Real*>(red));
            const double fa = 1.0 / (4 * kPi * rad * rad), fb = 3.0 / (8 * kPi * rad * rad * rad * rad);
            for (int c = 0; c < 3; ++c) {
                A[c] = double(la[c]) * fa;
                B[c] = double(la[3 + c]) * fb;
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
            if (a.mode == 3) {
                // first stage of the tensor-core operator: the Legendre stage runs in k_legendre_tc, which
                // reads one m at a time: stored m-major, [m][component][ring] complex
                float* fo = a.fg + a.fg_stride * s;
                for (int i = threadIdx.x; i < 6 * nt * P1; i += blockDim.x) {
                    const int m = i / (6 * nt), r = i - m * 6 * nt, c = r / (2 * nt), r2 = r - c * 2 * nt;
                    const int j = r2 >> 1, im = r2 & 1;
                    fo[i] = float(F[2 * (c * nt * P1 + j * P1 + m) + im]);
                }
                if (want_lop && threadIdx.x == 0)
                    for (int c = 0; c < 3; ++c) {
                        a.lop[6 * s + c] = A[c];
                        a.lop[6 * s + 3 + c] = B[c];
                    }
                return;
            }
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
    } else if (a.mode == 4) {
        // last stage of the tensor-core operator: the inverse-Legendre values (per ring and m) come from
        // k_legendre_tc, the rigid-mode vectors from the first stage
        const float* fi = a.fg + a.fg_stride * s;  // [m][component][ring] complex
        for (int i = threadIdx.x; i < 6 * nt * P1; i += blockDim.x) {
            const int m = i / (6 * nt), r = i - m * 6 * nt, c = r / (2 * nt), r2 = r - c * 2 * nt;
            const int j = r2 >> 1, im = r2 & 1;
            F[2 * (c * nt * P1 + j * P1 + m) + im] = Real(fi[i]);
        }
        if (want_lop)
            for (int c = 0; c < 3; ++c) {
                A[c] = a.lop[6 * s + c];
                B[c] = a.lop[6 * s + 3 + c];
            }
        __syncthreads();
    } else {
        for (int i = threadIdx.x; i < 6 * nc; i += blockDim.x) C[i] = Real(a.coef_in[2LL * g.coff[s] + i]);
        __syncthreads();
    }

    const bool do_inverse = a.mode == 2 || a.self_kind >= 0;
    if (do_inverse && a.mode != 4) {
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
            const Real b[3] = {sr * s0 * cp + stt * c0 * cp - sp * spp, sr * s0 * spp + stt * c0 * spp + sp * cp,
                               sr * c0 - stt * s0};
            Real ob[3];
            qrot(q, b, ob);
            o[0] = double(ob[0]);
            o[1] = double(ob[1]);
            o[2] = double(ob[2]);
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

// ---------------------------------------------------------------- Legendre stage on the tensor cores
// The FP32 sphere operator in three launches: k_sphere mode 3 (per sphere: rotation into the body
// frame, spherical components, DFT along phi, rigid-mode sums), k_legendre_tc (this kernel), k_sphere
// mode 4 (per sphere: inverse DFT, rotation back, self/identity/L terms). k_legendre_tc handles one
// order p, one m and a tile of up to kLegSpheres spheres of that order; the Legendre sums of all of
// them are two tcgen05 TF32 GEMMs (3xTF32 split, ~FP32 accuracy) with M = 128 rows = (sphere, kind):
//   forward  D_f[(s, k), n] = sum_K A_f[(s, k), K] B_f[n, K], K = (block b, ring j), b = 0, 1, 2 pairing
//            the weighted tables w_j P, w_j dP, w_j m Ps (n, m at ring j) with the phi-DFT values of the
//            radial, polar and azimuthal components so that row kind k = 0..5 gives directly
//            Re/Im of the radial coefficient, of the surface-gradient and of the toroidal coefficient
//            (times n(n+1)), e.g. Re g = sum_j Ft_re w dP + Fp_im w m Ps;
//   then, per (s, n), the self operator's multipliers (coefficients written out for the near field);
//   inverse  D_i[(s, k), j] = sum_K A_i[(s, k), K] B_i[j, K], K = (block b, n), the same pairing with the
//            unweighted tables: Re/Im of the radial, polar and azimuthal values at ring j.
// K runs in chunks of 32 through one shared-memory stage (operands built by the threads, B tables
// precomputed per (p, m) on the host in the operand layout of tc_sm100.h); accumulators in tensor
// memory (forward at column 0, inverse at column 64). The values of column m are read from and
// written back to the same per-sphere buffer fg ([m][component][ring] complex, so one m is contiguous).
// Waits are bounded; a timeout sets err.
constexpr int kLegSpheres = 21;   // spheres per tile: 6 rows each, 126 of the 128 MMA rows
constexpr int kLegK = 32;         // K per chunk
constexpr long long kLegWaitPolls = 1LL << 22;

__host__ __device__ inline int leg_kpad(int p) { return kLegK * ((3 * (p + 1) + kLegK - 1) / kLegK); }
__host__ __device__ inline int leg_npad(int n) { return 16 * ((n + 15) / 16); }

// value of the A operand row kind k (0..5) in block b (0..2) from the (Re, Im) pairs of three components
// v0, v1, v2 (radial / polar / azimuthal, or the radial / gradient / toroidal coefficients)
__device__ __forceinline__ float leg_a(int k, int b, float v0r, float v0i, float v1r, float v1i, float v2r, float v2i) {
    if (b == 0) return k == 0 ? v0r : (k == 1 ? v0i : 0.f);
    if (b == 1) return k == 2 ? v1r : (k == 3 ? v1i : (k == 4 ? v2r : (k == 5 ? v2i : 0.f)));
    // b == 2
    return k == 2 ? v2i : (k == 3 ? -v2r : (k == 4 ? -v1i : (k == 5 ? v1r : 0.f)));
}

__global__ void __launch_bounds__(128) k_legendre_tc(DevGeom g, int self_kind, float* __restrict__ fg,
                                                     long long fg_stride, float* __restrict__ coef_out) {
    const int4 T = g.leg_tiles[blockIdx.x];  // {order p, first entry in leg_sph, spheres, 0}
    const int p = T.x, m = blockIdx.y;
    if (m > p) return;
    const int nt = p + 1, nn = p + 1 - m, KP = leg_kpad(p), nch = KP / kLegK;
    const int NF = leg_npad(nn), NI = leg_npad(nt);
    const int cnt = T.z;
    extern __shared__ __align__(1024) unsigned char leg_smem[];
    unsigned char* sA = leg_smem;                     // A chunk hi | lo (2 x 16 KB)
    unsigned char* sB = leg_smem + 2 * 128 * kLegK * 4;  // B chunk hi | lo (N <= 48)
    __shared__ float sC[kLegSpheres][6][33];          // forward results (s, kind, n - m)
    __shared__ float sF[kLegSpheres][6 * 33];         // column m of the tile: [component][ring] complex
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        tc::tmem_alloc(&tbase, 128);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        tc::mbar_fence_init();
        s_fail = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    const int sl = tid / 6, kind = tid - 6 * (tid / 6);
    const int sph = sl < cnt ? g.leg_sph[T.y + sl] : 0;
    const bool row_ok = sl < cnt && (!g.active || g.active[g.prob[sph]]);
    // column m of every sphere of the tile (fg: per sphere [m][component][ring] complex), coalesced
    for (int i = tid; i < cnt * 6 * nt; i += 128) {
        const int s2 = i / (6 * nt), w = i - s2 * 6 * nt;
        sF[s2][w] = fg[fg_stride * g.leg_sph[T.y + s2] + (long long)m * 6 * nt + w];
    }
    __syncthreads();
    const float* tabs = g.leg_tab + g.leg_off[2 * (p * (kMaxOrder + 1) + m)];
    const float* tabi = g.leg_tab + g.leg_off[2 * (p * (kMaxOrder + 1) + m) + 1];
    unsigned phase = 0;

    // one GEMM: D[128 x N] at tensor-memory column dcol, A rows built by `arow(K index) -> value`,
    // B chunks from `tab` ([chunk][N x kLegK] in the operand layout)
    auto gemm = [&](int N, const float* tab, uint32_t dcol, auto&& arow) {
        for (int ch = 0; ch < nch; ++ch) {
            // B chunk: copy and split
            const float4* gb = reinterpret_cast<const float4*>(tab + (long long)ch * N * kLegK);
            for (int v = tid; v < N * kLegK / 4; v += 128) {
                const float4 b = __ldg(gb + v);
                float4 h, l;
                tc::tf32_split(b.x, h.x, l.x);
                tc::tf32_split(b.y, h.y, l.y);
                tc::tf32_split(b.z, h.z, l.z);
                tc::tf32_split(b.w, h.w, l.w);
                reinterpret_cast<float4*>(sB)[v] = h;
                reinterpret_cast<float4*>(sB + N * kLegK * 4)[v] = l;
            }
            // A chunk: this thread's row
#pragma unroll 2
            for (int q = 0; q < kLegK / 4; ++q) {
                float4 h, l;
                float v[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) v[e] = arow(ch * kLegK + 4 * q + e);
                tc::tf32_split(v[0], h.x, l.x);
                tc::tf32_split(v[1], h.y, l.y);
                tc::tf32_split(v[2], h.z, l.z);
                tc::tf32_split(v[3], h.w, l.w);
                const uint32_t off = tc::kmajor_offset(tid, 4 * q, kLegK);
                *reinterpret_cast<float4*>(sA + off) = h;
                *reinterpret_cast<float4*>(sA + 128 * kLegK * 4 + off) = l;
            }
            tc::fence_smem_async();
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t idesc = tc::idesc_tf32(128, N);
                const uint32_t a0 = tc::smem_u32(sA), al0 = a0 + 128 * kLegK * 4;
                const uint32_t b0 = tc::smem_u32(sB), bl0 = b0 + N * kLegK * 4;
                for (int ks = 0; ks < kLegK / 8; ++ks) {
                    const uint32_t o = ks * 256;
                    const uint64_t ah = tc::sdesc(a0 + o, 128, (kLegK / 4) * 128);
                    const uint64_t al = tc::sdesc(al0 + o, 128, (kLegK / 4) * 128);
                    const uint64_t bh = tc::sdesc(b0 + o, 128, (kLegK / 4) * 128);
                    const uint64_t bl = tc::sdesc(bl0 + o, 128, (kLegK / 4) * 128);
                    tc::mma_tf32(tmem + dcol, ah, bh, idesc, ch > 0 || ks > 0);
                    tc::mma_tf32(tmem + dcol, ah, bl, idesc, true);
                    tc::mma_tf32(tmem + dcol, al, bh, idesc, true);
                }
                tc::mma_commit(&mbar);
            }
            // the stage is refilled next: wait for this chunk's MMAs
            if (!tc::mbar_wait_bounded(&mbar, phase, kLegWaitPolls)) s_fail = 1;
            phase ^= 1;
            __syncthreads();
            if (s_fail) return false;
        }
        return true;
    };

    // ---- forward: A_f row (s, kind) = the phi-DFT values of column m at ring j (K = b * nt + j)
    auto arow_f = [&](int k) -> float {
        if (!row_ok || k >= 3 * nt) return 0.f;
        const int b = k / nt, j = k - b * nt;
        const float* f = sF[sl];
        return leg_a(kind, b, f[2 * j], f[2 * j + 1], f[2 * (nt + j)], f[2 * (nt + j) + 1], f[2 * (2 * nt + j)],
                     f[2 * (2 * nt + j) + 1]);
    };
    bool ok = gemm(NF, tabs, 0, arow_f);
    float d[64];
    if (ok) {
        tc::fence_after_sync();
        tc::tmem_ld_32x32b_x32(tmem + (uint32_t(warp * 32) << 16), *reinterpret_cast<float(*)[32]>(d));
        if (NF > 32) tc::tmem_ld_32x32b_x32(tmem + (uint32_t(warp * 32) << 16) + 32, *reinterpret_cast<float(*)[32]>(d + 32));
        tc::fence_before_sync();
        // coefficients of column m (times 1 / (n (n + 1)) for the gradient and toroidal parts)
        if (row_ok && tid < 6 * kLegSpheres) {
            const int nc = ncoef(p);
            const int blk = kind >> 1, im = kind & 1;
            for (int l = 0; l < nn; ++l) {
                const int n = m + l;
                const float inv = blk == 0 ? 1.f : (n > 0 ? 1.f / float(n * (n + 1)) : 0.f);
                const float v = d[l] * inv;
                sC[sl][kind][l] = v;
                if (coef_out) coef_out[2LL * g.coff[sph] + 2 * (blk * nc + cidx(n, m)) + im] = v;
            }
        }
        __syncthreads();
        // self operator multipliers per (s, n), in place (the formulas of k_sphere)
        for (int it = tid; it < cnt * nn; it += 128) {
            const int s2 = it / nn, l = it - s2 * nn, n = m + l;
            const float dn = float(n);
            float lh, lg, lx;
            if (self_kind == 0) {
                lh = dn / ((2 * dn + 1) * (2 * dn + 3));
                lg = (dn + 1) / ((2 * dn - 1) * (2 * dn + 1));
                lx = 1.f / (2 * dn + 1);
            } else if (self_kind == 4) {
                const float dh = 0.5f + 3.f / (2 * (2 * dn + 1) * (2 * dn + 3));
                const float dg = n == 1 ? 1.f : 0.5f - 3.f / (2 * (2 * dn - 1) * (2 * dn + 1));
                const float dx = n == 1 ? 1.f : 0.5f - 3.f / (2 * (2 * dn + 1));
                lh = 1.f / dh - 2;
                lg = 1.f / dg - 2;
                lx = 1.f / dx - 2;
            } else {
                lh = 3.f / (2 * (2 * dn + 1) * (2 * dn + 3));
                lg = -3.f / (2 * (2 * dn - 1) * (2 * dn + 1));
                lx = -3.f / (2 * (2 * dn + 1));
            }
            for (int c = 0; c < 2; ++c) {
                const float cr = sC[s2][c][l], cs = sC[s2][2 + c][l], cx = sC[s2][4 + c][l];
                const float h = (cr - dn * cs) * lh;
                const float gg = (cr + (dn + 1) * cs) / (2 * dn + 1) * lg;
                sC[s2][c][l] = h * ((dn + 1) / (2 * dn + 1)) + dn * gg;
                sC[s2][2 + c][l] = n > 0 ? (-h / (2 * dn + 1) + gg) : 0.f;
                sC[s2][4 + c][l] = n > 0 ? lx * cx : 0.f;
            }
        }
        __syncthreads();
        // ---- inverse: A_i row (s, kind) = the multiplied coefficients of column m (K = b * nt + n - m)
        auto arow_i = [&](int k) -> float {
            if (!row_ok || k >= 3 * nt) return 0.f;
            const int b = k / nt, l = k - b * nt;
            if (l >= nn) return 0.f;
            return leg_a(kind, b, sC[sl][0][l], sC[sl][1][l], sC[sl][2][l], sC[sl][3][l], sC[sl][4][l], sC[sl][5][l]);
        };
        ok = gemm(NI, tabi, 64, arow_i);
    }
    if (ok) {
        tc::fence_after_sync();
        tc::tmem_ld_32x32b_x32(tmem + (uint32_t(warp * 32) << 16) + 64, *reinterpret_cast<float(*)[32]>(d));
        if (NI > 32)
            tc::tmem_ld_32x32b_x32(tmem + (uint32_t(warp * 32) << 16) + 96, *reinterpret_cast<float(*)[32]>(d + 32));
        tc::fence_before_sync();
        if (row_ok && tid < 6 * kLegSpheres) {
            // kind -> (component, Re/Im) of the values at (ring j, m), doubled for m > 0
            const float e = m == 0 ? 1.f : 2.f;
            float* fo = fg + fg_stride * sph + (long long)m * 6 * nt;
            const int comp = kind >> 1, im = kind & 1;
            for (int j = 0; j < nt; ++j) fo[2 * (comp * nt + j) + im] = e * d[j];
        }
    } else if (tid == 0) {
        atomicExch(g.err, 2);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, 128);
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

constexpr size_t kLegDynSmem = 2 * 128 * kLegK * 4 + 2 * 48 * kLegK * 4;  // A and B chunk stages (44 KB)

// the FP32 sphere operator with its Legendre stage on the tensor cores (three launches)
int launch_sphere_tc(const DevGeom& g, SphereArgs a, cudaStream_t st) {
    a.fg = g.fgbuf;
    a.fg_stride = g.fg_stride;
    a.lop = g.lopbuf;
    a.mode = 3;
    k_sphere<float><<<g.N, kSphereThreads, sphere_smem<float>(g.pmax), st>>>(g, g.tab_f, a);
    k_legendre_tc<<<dim3(g.n_leg_tiles, g.pmax + 1), 128, kLegDynSmem, st>>>(g, a.self_kind, g.fgbuf, g.fg_stride,
                                                                           static_cast<float*>(a.coef_out));
    a.mode = 4;
    k_sphere<float><<<g.N, kSphereThreads, sphere_smem<float>(g.pmax), st>>>(g, g.tab_f, a);
    return 3;
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
    // 44 KB dynamic + 17 KB static shared memory: above the 48 KB a kernel gets without opting in
    cudaFuncSetAttribute(k_legendre_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kLegDynSmem));
    cudaFuncSetAttribute(k_sphere<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(sphere_smem<float>(kMaxOrder)));
    cudaFuncSetAttribute(k_sphere<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(sphere_smem<double>(kMaxOrder)));
}

int launch_sphere_op(const DevGeom& g, const double* x, double* out, double c_id, double c_self, int self_kind,
                     double c_lop, void* coef, bool fp32, cudaStream_t st) {
    SphereArgs a{x, nullptr, out, c_id, c_self, c_lop, self_kind, 0, coef};
    if (fp32 && g.sph_tc && self_kind >= 0 && g.n_leg_tiles > 0) return launch_sphere_tc(g, a, st);
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
