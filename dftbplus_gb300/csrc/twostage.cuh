// Two-stage symmetric tridiagonal reduction (dense -> band -> tridiagonal) and its back-transformation.
//
// The reference reaches two-stage reductions through ELPA (elecsolvers/elecsolvertypes.F90:27, the
// elpa solver) and MAGMA's dsygvd_m (math/eigensolver.F90:1143-1245); here they are written for one
// GB300:
//   stage 1 (sy2sb): panels of kBand columns are QR-factorised by one cooperative launch each (one
//            grid barrier per column, the panel resident in shared memory), and the trailing matrix
//            gets the two-sided update A22 <- Q^T A22 Q as GEMMs (symmetric product, rank-2*kBand
//            update of the lower triangle);
//   stage 2 (sb2st): the band is chased to tridiagonal form by one persistent cooperative kernel:
//            one CTA per sweep at a time, each sweep a chain of Householder tasks on kBand x kBand
//            blocks, sweep s running two tasks behind sweep s-1 (bounded waits on a progress word);
//   back-transformation: the bulge-chasing reflectors of kQ2Group consecutive sweeps at the same
//            chain position form one compact-WY block (a (kBand + kQ2Group - 1) x kQ2Group
//            parallelogram); the blocks are applied to column strips of Z, one CTA per strip; then
//            the stage-1 block reflectors as GEMMs.
// Eigenvectors of A = Q1 Q2 Z_tri: apply Q2 first, then Q1.
#pragma once
#include "gridsync.cuh"
#include "linalg.cuh"

namespace dg {

constexpr int kBand = 32;       // bandwidth of stage 1 (panel width)
constexpr int kQ2Group = 32;    // sweeps per compact-WY block of the stage-2 back-transformation

// Reduction used by the FP32 eigensolves of the mixed form (dftbgpu_set_two_stage): 0 one-stage
// panel tridiagonalisation, 1 two-stage, 2 (the default) two-stage from kTwoStageMinN orbitals on.
// Below that size the bulge chasing's chain of 2 n dependent tasks costs more than the one-stage
// panels (measured at n = 6,144: 289 ms against 220 ms per FP32 eigensolve).
extern std::atomic<int> g_twostage;
constexpr int kTwoStageMinN = 12000;
inline bool use_twostage(int n) {
  const int m = g_twostage;
  return m == 1 || (m == 2 && n >= kTwoStageMinN);
}

// Element offsets of the two-stage workspace (one buffer of T, integers at its end).
struct TwoStageLayout {
  int n = 0, kmax = 0, ngrp = 0, gmax = 0;
  size_t tau1 = 0, T1 = 0, X1 = 0, X = 0, X2 = 0, G = 0, G2 = 0, M = 0, split = 0, part = 0, top = 0, V2 = 0,
         tau2 = 0, T2 = 0, ints = 0, total = 0;   // in elements of T
  size_t split_elems = 0;
};
template <typename T>
TwoStageLayout twostage_layout(int n);
template <typename T>
size_t twostage_work_size(int n);

// Reduce the symmetric A (n x n, full symmetric storage on input; destroyed) to tridiagonal
// d[n], e[n-1]. V1 (n x n, ldv) receives the stage-1 reflectors; the workspace keeps the stage-1 T
// factors and the stage-2 reflectors for twostage_back. Bounded waits that give up raise *status
// to kDevIterCap.
template <typename T>
void twostage_reduce(cudaStream_t s, int n, T *A, int lda, T *d, T *e, T *V1, int ldv, T *work,
                     int *status);

// Z (n x k, ldz) <- Q1 Q2 Z: the eigenvectors of A from the tridiagonal eigenvectors in Z. A bounded
// wait that gives up raises *status to kDevIterCap.
template <typename T>
void twostage_back(cudaStream_t s, int n, int k, T *Z, int ldz, const T *V1, int ldv, T *work,
                   int *status = nullptr);

}  // namespace dg
