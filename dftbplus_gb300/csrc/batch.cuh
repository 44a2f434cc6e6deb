// Batched SCC-DFTB: thousands of independent small molecules (ragged sizes) solved together.
// One CTA owns one molecule for a whole SCC iteration (potentials, reduced Hamiltonian,
// Householder tridiagonalisation, implicit QL, Fermi filling, density matrix, Mulliken, Broyden):
// a molecule's n x n matrices (n <= kBatchMaxOrb) stay L2-resident while its CTA works on them.
#pragma once
#include "dftb_kernels.cuh"

namespace dg {

constexpr int kBatchThreads = 256;
constexpr int kBatchMaxOrb = 768;     // per molecule (tridiagonal and rotation vectors live in shared memory)
constexpr int kBatchMaxAtom = 1024;

// Per-molecule SCC state (device).
struct MolState {
  double nel, ef, eband, ts, e0, enonscc, escc, erep, err;
  int k;           // levels with non-zero filling
  int n_iter;      // SCC iterations done
  int mix_calls;   // Broyden mixing steps taken
  int conv;        // converged (FP64 iteration)
  int form;        // 0: FP64 eigensolve, 1: FP32 eigensolve, 2: perturbative update (mixed form)
  int status;      // DevStatus of the molecule (non-zero: failed, no further iterations)
  int verify;      // the next FP64 iteration checks a converged perturbative state (occupied vectors)
  int pert_run;    // perturbative iterations since the last reference
};

struct BatchDev {
  int nmol, natom, norb, M;         // M: Broyden history capacity (max SCC iterations)
  const int *order;                 // CTA -> molecule (largest first)
  const int *atom_off, *orb_off;    // [nmol + 1]
  const long long *mat_off;         // [nmol + 1] offsets of the per-molecule n x n matrices
  const long long *gam_off;         // [nmol + 1] offsets of the per-molecule nat x nat gamma
  const long long *pair_off;        // [nmol + 1] offsets of the per-molecule atom pairs (i < j)
  const int *a_orb;                 // [natom] global orbital offset of each atom
  const int *a_mol;                 // [natom] molecule of each atom
  const int *o_atom;                // [norb] atom of each orbital (global indices)
  const double *xyz;                // [3 natom]
  const int *species;               // [natom]
  // per-molecule matrices (column-major, leading dimension n of the molecule)
  double *H0, *S, *L, *Li, *A0, *A, *T, *Z, *rho;
  float *L32, *Li32, *A0_32, *A32, *T32, *Z32;
  // perturbative updates of the mixed form: reference C (all vectors) and X = S C in FP32, Mt / C dP
  // work arrays, reference density (FP64) and reference potentials (per atom)
  float *X32, *C32, *Mt32, *Zp32;
  double *rho_ref, *Vref;
  double *gam;                      // gamma matrix (1/r - short gamma, U on the diagonal)
  // per-orbital vectors
  double *eig, *fill, *dd, *ee;
  // per-atom vectors
  double *q0, *qin, *qout, *V, *Vout, *grad, *erep;
  double *dpair;                    // band-term gradient of each atom pair (3 per pair, for atom i)
  // Broyden (modified Broyden, one mixer per molecule): ww, aa, beta, cc per molecule (M, M^2, M^2,
  // M); dF, uu per molecule as nat x M blocks at atom_off * M; qlast, dlast per atom
  double *ww, *aa, *beta, *cc, *dF, *uu, *qlast, *dlast;
  MolState *st;
};

struct BatchOpts {
  double kT, tol, alpha, omega0, minw, maxw, wfac, net_charge, switch_tol;
  int max_iter, min_iter, mixed;
};

// Host-side batch state owned by a context.
struct BatchState {
  int nmol = 0, natom = 0, norb = 0, M = 0;
  long long nmat = 0, ngam = 0;
  size_t cap_atom = 0, cap_orb = 0, cap_mat = 0, cap_gam = 0, cap_mol = 0, cap_M = 0, cap_pair = 0;
  std::vector<int> h_atom_off, h_orb_off, h_species;
  std::vector<long long> h_mat_off;
  BatchDev d{};
  bool have_geom = false, have_scc = false, have_w = false;
  cudaGraphExec_t graph = nullptr;
  bool graph_mixed = false;
  int *d_active = nullptr;
  int *h_active = nullptr;           // pinned
  std::vector<void *> owned;         // geometry-sized buffers
  std::vector<void *> bro_owned;     // Broyden history (sized by max_iter)
};

// Geometry of all molecules: concatenated coordinates (3 x natom, Bohr) and species, atom_off[nmol+1].
// Builds H0/S, Cholesky factor and inverse, A0 = L^-1 H0 L^-T, gamma and repulsive energy per
// molecule. Returns a DFTBGPU_* status; msg receives an error description.
int batch_set_geometries(cudaStream_t s, BatchState &b, const ModelDev &m, const std::vector<SpeciesDev> &h_sp,
                         double cutoff, int nmol, const int *atom_off, const double *coords, const int *species,
                         bool coords_on_device, char *msg, size_t msg_len);
// SCC cycle of every molecule (lockstep iterations; converged molecules stop working).
int batch_scc(cudaStream_t s, BatchState &b, const ModelDev &m, const BatchOpts &o, char *msg, size_t msg_len);
// Energy gradients of every molecule after batch_scc (grad_dev: 3 x natom on the device).
int batch_gradients(cudaStream_t s, BatchState &b, const ModelDev &m, char *msg, size_t msg_len);
void batch_free(BatchState &b);

}  // namespace dg
