// DFTB-specific kernels (SK tables, electrostatics, filling, mixing, forces).
#pragma once
#include "common.cuh"

namespace dg {

struct ModelDev {
  int nsp;
  const SpeciesDev *sp;     // [nsp]
  const PairDev *pair;      // [nsp*nsp]
  const double *tab;        // SK tables (H and S), offsets in PairDev
  const double *rep;        // repulsive data
};

struct GeomDev {
  int natom;
  int norb;
  const double *xyz;        // [3*natom]
  const int *species;       // [natom]
  const int *orb_off;       // [natom+1]
};

// Device scalars written by the SCC kernels (index into a small double array).
enum Scalar : int {
  kSEf = 0, kSEband, kSTS, kSE0, kSEnonScc, kSEscc, kSErep, kSErr, kSNel, kSConv,
  kSNLevels, kSFermiStatus, kSDmu, kSCount = 16
};

// pair list
// Half neighbour list (i < j, r <= cutoff) in CSR order; fills pi/pj only if npairs <= cap.
void build_pairs(cudaStream_t s, const GeomDev &g, double cutoff, int *count, int *start, int *pi, int *pj,
                 size_t cap, int *npairs_host);
// H0 / S (dense, full symmetric)
void build_h0_s(cudaStream_t s, const ModelDev &m, const GeomDev &g, const int *start, const int *pj,
                int npairs, double *H0, double *S);
// repulsive energy (per atom, then summed into scal[kSErep])
void repulsive_energy(cudaStream_t s, const ModelDev &m, const GeomDev &g, double *eatom, double *scal);
// atom potential V = 1/r dq - gamma_short dq from atom populations q and reference q0
void potential(cudaStream_t s, const ModelDev &m, const GeomDev &g, const double *q, const double *q0,
               double *V);
// H = H0 + 1/2 S (V_mu + V_nu)
void assemble_h(cudaStream_t s, const GeomDev &g, const double *H0, const double *S, const double *V,
                double *H);
// DL = diag(V_orb) L (lower), for B = L^-1 DL
void reduced_shift(cudaStream_t s, const GeomDev &g, const double *L, const double *V, double *DL);
// A(lower) = A0 + 1/2 (B + B^T), B lower triangular
void add_half_lower(cudaStream_t s, int n, const double *A0, const double *B, double *A);
// FP32 versions and conversions for the reduced-precision iterations
void reduced_shift_f(cudaStream_t s, const GeomDev &g, const float *L, const double *V, float *DL);
void add_half_lower_f(cudaStream_t s, int n, const float *A0, const float *B, float *A);
void convert_d2f(cudaStream_t s, size_t n, const double *x, float *y);
void convert_f2d(cudaStream_t s, size_t n, const float *x, double *y);
void lower_f_to_sym_d(cudaStream_t s, int n, const float *A, double *B);
// First-order density-matrix perturbation around a reference eigen-decomposition (mixed form):
//   DC = diag(dV) C, DX = diag(dV) X with dV_l = V(atom l) - Vref(atom l)   (n x n, FP32)
void dmpt_scale(cudaStream_t s, const GeomDev &g, const double *V, const double *Vref, const float *C,
                const float *X, float *DC, float *DX);
//   Fermi-level shift dmu = sum_i f'_i M_ii / sum_i f'_i over i < k (into scal[kSDmu]); Mt is n x k
//   with Mt[j + i n] = M_ij
void dmpt_dmu(cudaStream_t s, int n, int k, const float *Mt, const double *fill, double kT, double *scal);
//   in place: Mt[j + i n] <- K_ij (M_ij - dmu delta_ij), halved for j < k (K = Fermi divided difference)
void dmpt_response(cudaStream_t s, int n, int k, float *Mt, const double *eig, const double *fill, double kT,
                   const double *scal);
//   B = Bref + D with D symmetric from its lower triangle (FP32), B full
void add_lower_f_sym_d(cudaStream_t s, int n, const double *Bref, const float *D, double *B);
// Fermi filling (spin unpolarised) from ascending eigenvalues; writes fill[n], scal[...]
void fermi_filling(cudaStream_t s, int n, const double *eig, double nel, double kT, double *fill,
                   double *scal);
// Mulliken populations per orbital and atom + Tr(rho H0) into scal[kSEnonScc]
void mulliken(cudaStream_t s, const GeomDev &g, const double *rho, const double *S, const double *H0,
              double *qorb, double *qatom, double *eorb, double *scal);
// E_SCC = 1/2 sum V_A dq_A
void scc_energy(cudaStream_t s, int natom, const double *V, const double *q, const double *q0, double *scal);
// Broyden mixing on device (single CTA); returns nothing, writes scal[kSErr], scal[kSConv], qin.
struct BroydenDev {
  int max_iter;
  double *ww, *aa, *dF, *uu, *qlast, *dlast;
};
void broyden_step(cudaStream_t s, int natom, int it, int mix_it, int min_iter, int max_iter_scc, double tol,
                  double alpha, double omega0, double minw, double maxw, double wfac,
                  BroydenDev b, double *qin, const double *qout, double *scal);
// gradients
void gradient_bands(cudaStream_t s, const ModelDev &m, const GeomDev &g, const double *rho,
                    const double *W, const double *V, double *grad);
void gradient_dc_rep(cudaStream_t s, const ModelDev &m, const GeomDev &g, const double *q,
                     const double *q0, double *grad);
// Parameter adjoints of the converged state (adjoint.cu): dE/d(table values) accumulated into
// dham/dover (layout of the uploaded sk_ham/sk_over, zeroed by the caller) and dE/dU per species.
void sk_adjoint(cudaStream_t s, const ModelDev &m, const GeomDev &g, const int *pi, const int *pj, int npairs,
                const double *rho, const double *W, const double *V, double *dham, double *dover);
void hubbard_adjoint(cudaStream_t s, const ModelDev &m, const GeomDev &g, const double *q, const double *q0,
                     double *dU);
void energy_weights(cudaStream_t s, int k, const double *fill, const double *eig, double *fe);

}  // namespace dg
