// sh_host.h — host-side spectral precompute for the device kernels (per SH order p):
// Gauss-Legendre rings, normalized associated Legendre tables, DFT twiddles, the
// irregular-solid-harmonic recurrence coefficients and the sparse linear maps from a
// sphere's vector-SH coefficients to the coefficient sets of its exterior Laplace
// potentials (used by the near-field evaluation).
#pragma once
#include <complex>
#include <vector>

namespace smob {

struct HostOrderTables {
    int p = 0, nt = 0, nphi = 0, nc = 0;
    std::vector<double> ct, st, wq;      // rings north -> south: cos, sin, quadrature weight (unit sphere)
    std::vector<double> cph, sph;        // cos/sin of phi_k
    std::vector<double> cosmk, sinmk;    // [m*nphi + k], m <= p
    std::vector<double> P, dP, Ps;       // [j*nc + cidx(n,m)]
};

// sparse map in CSR: rows are (idx(n,m) of degree <= p+3) x set x (re,im), interleaved as
// row = (idx * nsets + set) * 2 + reim; columns index the real view of the 3*ncoef(p)
// complex VSH coefficients (col = 2*(block*ncoef(p) + idx) + reim).
struct SparseMap {
    int rows = 0, cols = 0, nsets = 0;
    std::vector<int> rowptr, col;
    std::vector<double> val;
};

const HostOrderTables& host_tables(int p);
// VSH coefficients (3 blocks of ncoef(p) complex values) evaluated at one body-frame direction
// (0 < theta < pi); Cartesian body-frame vector out[3]
void vsh_eval_point(int p, const std::complex<double>* c, double theta, double phi, double* out);
void gauss_legendre_nodes(int n, std::vector<double>& x, std::vector<double>& w);
// trac = true: 25 sets (div L, Hessians of L_x, L_y, L_z, L_r); false: 15 sets (L_j, grad L_j, grad L_r)
const SparseMap& near_map(int p, bool trac);
// unit-sphere grid nodes of order p (ring-major, as the sphere grids): [node][3]
void unit_nodes(int p, std::vector<double>& xyz);
// FP32 map from the weighted grid sources of an order-p sphere to equivalent sources on its order-pe
// grid (pe < p), transposed: [j (fine node)][k (coarse node)]
const std::vector<float>& coarse_map(int p, int pe);
const std::vector<double>& coarse_map_d(int p, int pe);
// recurrence coefficients of the irregular solid harmonics up to degree nmax:
// c1[cidx(n,m)] = (2n+1)/sqrt((n+1)^2-m^2), c2[cidx(n,m)] = sqrt((n^2-m^2)/((n+1)^2-m^2)), diag[m] = sqrt((2m-1)/(2m))
void theta_recurrence(int nmax, std::vector<double>& c1, std::vector<double>& c2, std::vector<double>& diag);

}  // namespace smob
