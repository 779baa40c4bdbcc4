// smob_internal.h — device data layout and kernel entry points of libsmob.
//
// Layout in HBM (one context = one batch of independent problems):
//   spheres  : centre[3N], radius[N], quat[4N] (w,x,y,z), order[N], gidx/glen (point range),
//              coff (coefficient offset, complex units), prob[N]
//   points   : coords/norms[3M] (FP64 lab frame), weights[M], sid[M];
//              pos32/nrm32 float4 (x,y,z relative to the problem's origin, w = sphere id bits);
//              pos64/nrm64 double4_32a (same, FP64)
//   near     : CSR by target sphere (nbr_start[N+1], nbr_src[pairs], sorted by source)
//   far field: work items (target block x source-sphere chunk) and a partial-sum buffer
//              laid out per problem as [chunk][point][3] (deterministic fixed-order reduction)
//   tables   : per SH order p: Legendre tables at the Gauss-Legendre rings, DFT twiddles,
//              and the sparse linear maps from VSH coefficients to the near-field coefficient sets
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

struct smob_ctx;

namespace smob {

constexpr int kMaxOrder = 32;
constexpr int kFarThreads = 128;         // far-field CTA size (FP32: 1, 2 or 4 targets per thread)
constexpr int kFarThreadsDF = 32;        // float-float far-field CTA (2 packed targets per thread: 64 targets)
constexpr int kFarTargets32 = 256;       // targets per FP32 far-field work item
constexpr int kFarTargets64 = 128;       // targets per FP64 far-field work item
constexpr int kFarTile = 256;            // sources staged per shared-memory tile (FP64 / float-float)
constexpr int kFarTile32 = 640;          // FP32 tile: a whole p <= 16 sphere (578 points) in one round
constexpr int kRepTile = 256;            // several-RHS FP32 tile (positions + up to 8 source columns)
constexpr int kRepTileDF = 128;          // several-RHS float-float tile (hi/lo positions + up to 4 columns)
constexpr int kSphereThreads = 256;      // per-sphere transform CTA
constexpr int kNearThreads = 128;        // near-field CTA (one target point per thread)
constexpr int kVecChunk = 4096;          // segmented reduction chunk (elements), never crosses a problem
constexpr int kNearSetsTrac = 25;        // div L, Hessians of L_x,L_y,L_z,L_r
constexpr int kNearSetsSL = 15;          // L_j, grad L_j, grad L_r
constexpr int kNearTcChunk = 16;         // harmonics (complex) per K chunk of the tensor-core near field
// floats per near-source slot of the tiled FP32 sets (the B operand of the tensor-core near field):
// chunks of kNearTcChunk harmonics up to degree pmax + 3, each a (32 or 16) x 2 kNearTcChunk tile
inline long long near_tile_stride(int pmax, bool trac) {
    const int nck = ((pmax + 4) * (pmax + 5) / 2 + kNearTcChunk - 1) / kNearTcChunk;
    return (long long)nck * (trac ? 32 : 16) * 2 * kNearTcChunk;
}
constexpr int kCoarseLevels = 8;         // coarse equivalent-source levels per sphere (FP32 far field)
constexpr int kCoarseTileNodes = 32;     // coarse nodes per CTA of the coarse-strength GEMMs (multiple of 16)
constexpr int kCoarseTcNodes = 128;      // tensor-core coarse-strength GEMM: coarse nodes (MMA rows) per CTA
constexpr int kCoarseTcSph = 16;         // and spheres per CTA (three MMA columns each)
constexpr int kCoarseTcSplit = 4;        // CTAs per tile, each a quarter of the K chunks
// interpolation tiles of the coarse targets (the host lists at most this many entries per tile; the
// kernels k_ct_interp / k_ct_interp_df read exactly these): FP32 set 2 entries x 128 grid points,
// float-float set 1 entry x 256 grid points (two per thread)
constexpr int kCiEnt = 2, kCiPts = 128;
constexpr int kCiEntD = 1, kCiPtsD = 256;

__host__ __device__ inline int ncoef(int p) { return (p + 1) * (p + 2) / 2; }
__host__ __device__ inline int cidx(int n, int m) { return n * (n + 1) / 2 + m; }

// per-order table descriptor (offsets into the table buffers, in elements)
struct OrderTables {
    int p, nt, nphi, nc;
    int ring;        // offset of ct, st, wq arrays (nt each) in tab_d
    int leg;         // offset of P, dP, Ps arrays (nt*nc each) in tab_d
    int twiddle;     // offset of cos(m phi_k), sin(m phi_k) [(p+1)*nphi each] in tab_d
    int cph;         // offset of cos(phi_k), sin(phi_k) [nphi each] in tab_d
    int trac_map;    // offset into sparse map arrays (row pointer base), -1 if absent
    int sl_map;
    int trac_rows, sl_rows;  // rows = 2 * sets * ncoef(p+3)
};

struct FarItem {
    int t0, t1;      // target point range (one problem)
    int s0, s1;      // source sphere range (one problem)
    int problem;
    int chunk;       // chunk index within the problem
};

struct Problem {
    int s0, s1;      // spheres
    int p0, p1;      // points
    int nchunks;     // far-field source chunks
    long long poff;  // partial-buffer offset (elements of 3-vectors * chunks)
    int v0, v1;      // vector element range [3*p0, 3*p1)
    int c0, c1;      // reduction chunk range (segmented dots)
};

// coarse equivalent sources of one tolerance (see DevGeom)
struct CoarseSet {
    int ncent;                 // (sphere, level) entries
    float clog_eps, cmargin;
    const int4* clev;          // [N][kCoarseLevels] {pe (0: unused), first coarse point, count, map offset}
    const int2* cent;          // [ncent] {sphere, level}
    const float4* cpos32;      // coarse points: x, y, z relative to the problem origin, w = sphere id bits
    const float4* cpos32lo;    // float-float set: the coordinates' low parts
    const float* cmap;         // FP32 set: coarse maps, [fine node][coarse node] per (p, pe)
    const float2* cmapf2;      // float-float set: the same maps as (hi, lo) float pairs
    float4* csrc;              // strengths of the current pass (float-float set: hi, lo interleaved)
    int crep;                  // coarse points of one replica (several-RHS contexts; else all of them)
    // the strengths as small GEMMs, one per (p, pe) map: CTA tiles of kCoarseTileNodes coarse nodes x 8 spheres
    int ncdesc;
    const int4* cdesc;         // [ncdesc] {group, first coarse node, first entry in gent, entries (<= 8)}
    const int4* cgrp;          // per group {map offset, fine nodes N_g(p), coarse nodes N_e(pe), 0}
    const int2* gent;          // entries grouped by map: {sphere, first coarse point of that sphere's level}
    // the same GEMMs on the tensor cores (FP32 set): tiles of 128 coarse nodes x 16 spheres
    int ncdesc_tc;
    const int4* cdesc_tc;      // [ncdesc_tc] {group, first coarse node, first entry in gent, entries (<= 16)}
    const float4* cmapA;       // their A operand, pre-split and tiled per group (offset cgrp.w, in floats)
    float4* cpart;             // [kCoarseTcSplit][ncoarse32] partial strengths of the K splits
    unsigned* ctile_count;     // [ncdesc_tc] splits finished per tile (zero between launches)
    long long ncoarse32;       // coarse points of the set
    // Coarse targets: a target sphere t takes the far field of a well-separated source sphere s at the
    // nodes of one of its own coarse levels and interpolates it to its grid (the transposed map);
    // level: the coarsest built pe with pe >= clog_eps / log(a_t / (|c_t - c_s| - a_s)) + ctmargin, if
    // it has at most kCoarseTargetNum / kCoarseTargetDen of the sphere's grid points (else the pair
    // stays on the grid targets). FP32 set: FP32 passes; float-float set: the fused float-float pass
    // (traction and single layer).
    int ctgt;                  // 1: coarse targets on
    float ctmargin;
    const float4* cnrm32;      // coarse node normals, w = level index bits (float-float set: high parts)
    const float4* cnrm32lo;    // float-float set: the normals' low parts
    const float* cmapT;        // FP32 set: the maps transposed, [coarse node][fine node], at the maps' offsets
    const float2* cmapTdf;     // float-float set: the same from the FP64 maps as (hi, lo) float pairs
    const int* ctused;         // [N][kCoarseLevels]: the entry is a listed coarse-target entry (CtEnt)
    int nctent;
    const struct CtEnt* ctent; // listed and grid entries
    const int* ctsrc;          // the entries' candidate source spheres
    int2* ctcand;              // per candidate, from the geometry (launch_ct_classify): the first point and
                               // count of the sources it is read from (count < 0: coarse points, -count of
                               // them; 0: not this entry's pair)
    float4* ctu;               // FP32 set: far field at the coarse targets of the current pass
    float* ctinterp;           // FP32 set: [kCoarseLevels + 1][M][3]: listed entries interpolated to the
                               // grid by level slot, and the grid entries' sums
    double* ctud;              // float-float set: traction and single layer at the coarse targets [6]
    double* ctinterpd;         // float-float set: as ctinterp with [6] per point
    int nctitile_tc;           // FP32 set: the tensor-core interpolation's tiles (CtITile with mapoff = the A
    const struct CtITile* ctitile_tc;  // tile group's offset in cmapI, up to 16 entries), entry lists, and
    const int* ctient_tc;      // the maps [grid point][coarse node] pre-split and tiled as its A operand
    const float4* cmapI;
    int nctitile;              // interpolation tiles (CtITile) and their entry lists
    const struct CtITile* ctitile;
    const int* ctient;
};

// coarse targets of a sphere: at most 7/10 of its grid points (interpolation plus coarse evaluation
// must undercut the grid evaluation)
constexpr int kCoarseTargetNum = 7, kCoarseTargetDen = 10;

// A listed coarse-target entry (sphere t, level l): its nodes are the coarse points [q0, q0 + n) of
// the set, its candidate sources ctsrc[src0, src0 + nsrc) (every s with tgt_level(t, s) == l and
// neighbours of the level boundary; the kernels check the rule per pair); partial sums at poff as
// [chunk][node][3]. A grid entry (l = -1, one per sphere) has the sphere's grid points [q0, q0 + n)
// as nodes and the sources whose pair stays on the grid targets (tgt_level == -1) as candidates;
// its sums go to slot kCoarseLevels of ctinterp.
struct CtEnt {
    int t, l, q0, n;
    int src0, nsrc, nchunks, problem;
    long long poff;
    long long pad;
};

// one coarse-target work item: nodes [k0, k0 + nb) of entry ent in a block of w nodes (FP32: 128 ... 8,
// one per thread of a slice, 128 / w slices share the sources; float-float set: 64 ... 4, two per thread,
// 64 / w slices) against candidates [sa, sb) of the entry, partial chunk
struct CtWork {
    int ent, k0, nb, w;
    int sa, sb, chunk, pad;
};

// one interpolation tile: grid points [j0, j0 + 128) of up to 2 listed entries (float-float set: 256, 1)
// sharing one map (order p, level pe): entries ctient[e0, e0 + ne), map at mapoff ([n][ng])
struct CtITile {
    int mapoff, ng, n, e0;
    int ne, j0, pad0, pad1;
};

struct DevGeom {
    int N, M, P;
    int pmax;             // largest SH order present (sizes shared memory of the per-sphere kernels)
    int near_lanes;       // lanes per target point in the near-field kernel (1, 2, 4 or 8)
    int near_tc;          // FP32 near field on the tensor cores (k_near_eval_tc, tiled sets); 0: SIMT kernel
    int coarse_tc;        // FP32 coarse-target interpolation on the tensor cores (k_ct_interp_tc)
    // FP32 sphere operator with the Legendre stage on the tensor cores (k_legendre_tc; 0: one SIMT kernel):
    // tiles {order p, first entry of leg_sph, spheres (<= 21), 0} of spheres of one order; B operand
    // tables per (p, m), forward and inverse, at leg_off[2 (p (kMaxOrder + 1) + m) + {0, 1}] floats into
    // leg_tab; per-sphere workspaces fgbuf (fg_stride floats: [3][p+1][p+1] complex) and lopbuf (6 doubles)
    int sph_tc;
    int n_leg_tiles;
    const int4* leg_tiles;
    const int* leg_sph;
    const float* leg_tab;
    const int* leg_off;
    float* fgbuf;
    long long fg_stride;
    double* lopbuf;
    int* err;             // device error word: kernels whose bounded waits gave up set it (0: none)
    int th_c1, th_c2, th_diag;  // offsets of the irregular-solid-harmonic recurrence tables in tab_d/tab_f
    const double* center;
    const double* radius;
    const double* quat;   // always present (identity filled in)
    const int* order;
    const int* gidx;
    const int* glen;
    const int* coff;      // complex offset of each sphere's 3*ncoef(p) coefficients
    const int* prob;
    const double* coords;
    const double* norms;
    const double* weights;
    const int* sid;
    const float4* pos32;
    const float4* nrm32;
    const float4* pos32lo;  // float-float low parts: coordinate - float(coordinate), normal likewise
    const float4* nrm32lo;
    const double4_32a* pos64;
    const double4_32a* nrm64;
    const int* nbr_start;
    const int* nbr_src;
    const unsigned char* nbr_precise;  // per pair: surface gap < 0.1 * min radius (evaluated in FP64 in mixed mode)
    const int* near_src_slot;  // per sphere: slot in the near-set buffer, -1 if not a near source
    const Problem* problems;
    const OrderTables* tabs;   // indexed by p (kMaxOrder+1 entries)
    const double* tab_d;
    const float* tab_f;
    const int* map_rowptr;     // sparse maps (CSR, rows within a map are contiguous)
    const int* map_col;
    const double* map_val_d;
    const float* map_val_f;
    const unsigned char* active;  // per problem: operator work enabled
    // Far field from coarse equivalent sources for well-separated sphere pairs: one set for the FP32
    // passes and one, with a tighter tolerance, for the float-float passes (ncent = 0: off). A source
    // sphere s has up to kCoarseLevels coarse orders pe, ascending; a target sphere t may use the
    // coarsest with pe >= clog_eps / log(a_s / (|c_t - c_s| - a_t)) + cmargin.
    CoarseSet cs32, cshp;
    const float4* sph32;       // per sphere: centre relative to the problem origin (FP32), radius
    const double* cnode;       // unit nodes of the coarse orders, [node][3]
    const int* cnode_off;      // [kMaxOrder + 1] first node of order pe in cnode
};

// ---------------------------------------------------------------- kernels (launch wrappers)
// Every wrapper launches on `st` and returns the number of kernels it launched.
// Far field: out[3M] += sum over far sources of c_sl*S + c_trac*K(dot n_target).
int launch_far_pack(const DevGeom& g, const double* x, double c, float4* src32, double4_32a* src64, bool fp32,
                    cudaStream_t st);
// coarse equivalent-source strengths of this pass from the FP32 grid sources (before every FP32
// launch_far_field when g.ncent > 0)
int launch_coarse_src(const DevGeom& g, const float4* src32, cudaStream_t st);
// the FP32 coarse strengths as 3xTF32 GEMMs on the tcgen05 tensor cores (cs32.cdesc_tc tiles); a tile
// that gave up waiting for its MMAs sets *g.err and writes nothing
int launch_coarse_src_tc(const DevGeom& g, const float4* src32, cudaStream_t st);
// the float-float set's strengths (hi, lo) from the float-float grid sources of launch_far_pack_df
int launch_coarse_src_df(const DevGeom& g, const float4* src2, cudaStream_t st);
// tpt: FP32 targets per thread (1, 2 or 4); FP32 items must cover kFarThreads * tpt targets
int launch_far_field(const DevGeom& g, const FarItem* items, int nitems, bool trac, bool fp32, const float4* src32,
                     const double4_32a* src64, void* partial, cudaStream_t st, int tpt = 2);
// ct: 0 the chunks' sums of partial; 1 (FP32 with coarse targets) the grid entries' sums and the
// listed entries' interpolated values from cs32.ctinterp instead (partial is not read); 2 / 3 the same
// from cshp.ctinterpd, traction / single layer (the fused float-float pass)
int launch_far_reduce(const DevGeom& g, const void* partial, bool fp32, double pre, double* out, cudaStream_t st,
                      int ct = 0);
// FP32 far field with coarse targets (after launch_coarse_src): the work items of the listed and the
// grid entries into partial (CtEnt layout), their chunks summed into cs32.ctu (listed) and the grid
// slot of cs32.ctinterp (grid entries), and the listed entries interpolated to their spheres' grids
// into their level slots (launch_far_reduce with ct = 1 adds the slots)
int launch_far_ct(const DevGeom& g, const CtWork* works, int nworks, bool trac, const float4* src32, float* partial,
                  cudaStream_t st);
// per geometry (after launch_coarse_grid): every entry's candidates resolved by tgt_level and level_bit
// into cs.ctcand, which the target kernels read instead of evaluating the rules per pass
int launch_ct_classify(const DevGeom& g, const CoarseSet& cs, cudaStream_t st);
// the fused float-float pass (traction and single layer) with the float-float set's coarse targets
// (after launch_coarse_src_df): as launch_far_ct, into cshp.ctud / ctinterpd (launch_far_reduce with
// ct = 2 and 3 adds the slots)
int launch_far_df_ct(const DevGeom& g, const CtWork* works, int nworks, const float4* src2, double* partial,
                     cudaStream_t st);
// coarse points of every (sphere, level) entry of a set, relative to the problem origins (after
// launch_regrid); cpos32lo (may be null) receives the low parts
int launch_coarse_grid(const DevGeom& g, const CoarseSet& cs, const double* org, float4* cpos32, float4* cpos32lo,
                       float4* cnrm32, float4* cnrm32lo, cudaStream_t st);
// FP32 far field of nrep replicas of one problem (replica r = problem r, points [r*rep_M, (r+1)*rep_M)):
// items are replica 0's (kFarThreads targets each); each pair's geometry serves all replicas
int launch_far_field_rep(const DevGeom& g, const FarItem* items, int nitems, int nrep, int rep_M, bool trac,
                         const float4* src32, float* partial, cudaStream_t st);
// float-float far field (hi/lo float pairs on the FP32 pipe); partial sums in FP64 (the FP64 buffer).
// Items cover 2 * kFarThreadsDF targets. kind: 0 single layer, 1 traction (both into partial),
// 2 traction into partial and single layer into partial_sl from the same sources in one pass.
int launch_far_pack_df(const DevGeom& g, const double* x, double c, float4* src2, cudaStream_t st);
int launch_far_field_df(const DevGeom& g, const FarItem* items, int nitems, int kind, const float4* src2,
                        double* partial, double* partial_sl, cudaStream_t st);
// the fused float-float pass (traction -> partial, single layer -> partial_sl) for nrep replicas of one
// problem; items are replica 0's (kFarThreads targets each)
int launch_far_field_df_rep(const DevGeom& g, const FarItem* items, int nitems, int nrep, int rep_M,
                            const float4* src2, double* partial, double* partial_sl, cudaStream_t st);

// Per-sphere operator: out += c_id*x + c_self*Self[x] + c_lop*L[x]; coefficients of x written to coef
// (self_kind: -1 none, 0 single layer, 3 traction principal value, 4 inverse of the sphere's own
// I/2 + K_PV + L minus 2 I, used with c_id = 2 as the block-diagonal preconditioner).
int launch_sphere_op(const DevGeom& g, const double* x, double* out, double c_id, double c_self, int self_kind,
                     double c_lop, void* coef, bool fp32, cudaStream_t st);
void configure_sphere_kernels();
void configure_near_kernels();  // shared-memory limits of the staged near-field kernels
// Transforms only: coef (double) from grid (g2s), or grid from coef (s2g, overwrite)
int launch_sh_g2s(const DevGeom& g, const double* grid, double* coef, cudaStream_t st);
int launch_sh_s2g(const DevGeom& g, const double* coef, double* grid, cudaStream_t st);

// Near field: sets from coefficients (per near source sphere), then spectral evaluation per target sphere.
// FP32 with g.near_tc: the sets are written as the tiles of the tensor-core kernel at stride
// near_tile_stride(g.pmax, trac) per slot (`stride` is then not used); the buffer's padding must be zero.
// df (FP64 coefficients only): the sets as float pairs (hi, lo) for the float-float evaluation
int launch_near_sets(const DevGeom& g, const void* coef, bool trac, bool fp32, void* sets, int nslots,
                     const int* slot_sphere, long long stride, cudaStream_t st, bool df = false);
// pair_filter: 0 all near pairs, 1 pairs with gap >= 0.1 min radius, 2 the near-singular pairs only;
// df (with fp32 false and float-pair sets): the float-float kernel instead of the FP64 one
int launch_near_eval(const DevGeom& g, const void* sets, long long stride, bool trac, bool fp32, double c, double* out,
                     cudaStream_t st, int pair_filter = 0, bool df = false);

// Neighbour list on the device (nbrlist.cu): near pairs of every problem by the reference's rule
// 0 < |c_s - c_t|^2 < (1.5 a_s + 1.5 a_t)^2 (problems[].s0/s1 and prob give each sphere's problem).
// count: near sources per target; scan: CSR offsets start[N+1], near-source slots slot_of[N] (-1 if
// none), totals {pairs, slots}; fill: sources (ascending per target), near-singular flags, slot_sphere.
int launch_nbr_count(const double* centers, const double* radii, const int* prob, const Problem* problems, int N,
                     int* count, cudaStream_t st);
int launch_nbr_scan(const int* count, int N, int* start, int* slot_of, int* totals, cudaStream_t st);
int launch_nbr_fill(const double* centers, const double* radii, const int* prob, const Problem* problems, int N,
                    const int* start, const int* slot_of, int* src, unsigned char* precise, int* slot_sphere,
                    cudaStream_t st);
// first overlapping or touching pair (t * N + s, s > t, same problem) by atomicMin into *first
int launch_overlap_check(const double* centers, const double* radii, const int* prob, const Problem* problems, int N,
                         unsigned long long* first, cudaStream_t st);

// Geometry update: grid points, normals and far-field copies from the current centres/orientations
// (org: 3 per problem); writes the buffers that g's read-only views point to
int launch_regrid(const DevGeom& g, const double* org, cudaStream_t st);

// Rigid-body pieces of the mobility solve
int launch_rigid_density(const DevGeom& g, const double* force6n, double* rho, cudaStream_t st);
int launch_rigid_average(const DevGeom& g, const double* u, double inv_visc, double* vel6n, cudaStream_t st);

// Host view of a context's spheres and grid for the file writers (the grid is refreshed from the
// device first if a geometry update changed it)
struct HostSpheres {
    int N = 0, M = 0;
    const double *centers = nullptr, *radii = nullptr, *quats = nullptr, *coords = nullptr, *weights = nullptr;
    const int *orders = nullptr, *gidx = nullptr;
};
HostSpheres host_spheres(const ::smob_ctx* c);


}  // namespace smob
