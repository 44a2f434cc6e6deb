// Dense linear algebra on one GB300 (column-major, device pointers, one stream). The eigensolver
// pieces are templates on the scalar type: FP64 for the plain path, FP32 for the reduced-precision
// SCC iterations of the mixed form. Cholesky and L^-1 are FP64 only.
#pragma once
#include <atomic>

#include "common.cuh"

namespace dg {

// Triangular structure hints for GEMM (zero regions are skipped, not read).
enum GemmFlags : int {
  kALower = 1,   // op(A)[i][p] == 0 for p > i
  kAUpper = 2,   // op(A)[i][p] == 0 for p < i
  kBLower = 4,   // op(B)[p][j] == 0 for p < j
  kBUpper = 8,   // op(B)[p][j] == 0 for p > j
  kCLower = 16,  // only tiles touching the lower triangle (i >= j) are computed
};

// C = alpha * op(A) * op(B) + beta * C ; op = 'N' or 'T'. m, n, k >= 0.
// With a workspace (work_elems elements) a GEMM whose output has fewer than kSplitTarget 64x64
// tiles and K >= 1024 is split along K (deterministic reduction). Without one, nothing is split.
constexpr long long kSplitTarget = 2 * 152;
template <typename T>
void gemm(cudaStream_t s, char ta, char tb, int m, int n, int k, T alpha, const T *A, int lda, const T *B,
          int ldb, T beta, T *C, int ldc, int flags = 0, T *work = nullptr, size_t work_elems = 0);
// Tensor-core product for FP32 operands (tc_gemm.cu): split-BF16 compensated products on tcgen05
// with FP32 accumulation in TMEM; same arguments and flags as gemm. Returns a cudaError_t value.
int tc_gemm(cudaStream_t s, char ta, char tb, int m, int n, int k, float alpha, const float *A, int lda,
            const float *B, int ldb, float beta, float *C, int ldc, int flags);
// Non-zero if a tensor-core GEMM timed out on a bounded wait since the last call (flag cleared).
int tc_gemm_error();
// When set, the perturbative updates of the mixed form use tc_gemm. Their operands carry the
// potential change only, so the tensor cores' accumulation (not IEEE round-to-nearest over long K)
// is scaled down by it; full FP32 eigensolves keep FP32 FMA products.
extern std::atomic<bool> g_tc_gemm;   // process-wide switch

// FP64-class product on the tensor cores (tc_dgemm.cu): exact BF16 digit-slice products (eight
// 7-bit digits per element, integer accumulation), same arguments and flags as gemm. Returns a
// cudaError_t value. tc_dgemm_reserve sizes its workspace ahead of use.
int tc_dgemm(cudaStream_t s, char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
             const double *B, int ldb, double beta, double *C, int ldc, int flags);
int tc_dgemm_reserve(int m, int n, int k);
double tc_dgemm_estimate_s(int m, int n, int k);   // seconds, for routing
int tc_dgemm_error();
// While g_tc_dgemm is set, gemm<double> sends products with m, n >= 64 and k >= 32 to tc_dgemm
// where a cost estimate favours it (the mixed form sets it around its FP64 iterations when
// g_tc_dgemm_mixed allows it).
extern thread_local bool g_tc_dgemm;        // per calling thread
extern std::atomic<bool> g_tc_dgemm_mixed;  // process-wide switch
// Kernel of tc_dgemm (process-wide): 0 (default) the single-stage kernel (one 64-wide K block per
// round trip of copies, MMAs and readback); 1 pipelined, TMA-fed, windowed TMEM readback.
extern std::atomic<int> g_dg_kernel;

// FP32-class product on the tensor cores (tc_fgemm.cu): exact BF16 digit-slice products (three
// signed 8-bit digits per element, six products, integer accumulation), same arguments and flags as
// gemm. Returns a cudaError_t value. While g_tc_fgemm is set, gemm<float> sends products with m, n, k
// >= 512 there (the mixed form sets it around its FP32 eigensolves when g_tc_fgemm_mixed allows it).
int tc_fgemm(cudaStream_t s, char ta, char tb, int m, int n, int k, float alpha, const float *A, int lda,
             const float *B, int ldb, float beta, float *C, int ldc, int flags);
int tc_fgemm_error();
extern thread_local bool g_tc_fgemm;        // per calling thread
extern std::atomic<bool> g_tc_fgemm_mixed;  // process-wide switch

void dgemm(cudaStream_t s, char ta, char tb, int m, int n, int k, double alpha, const double *A,
           int lda, const double *B, int ldb, double beta, double *C, int ldc, int flags = 0,
           double *work = nullptr, size_t work_elems = 0);

// Optional timing of every GEMM launch (events around each launch, executed FLOPs counted from
// the tile k-ranges the kernel actually iterates). Enabled by the context's profiler; launches
// recorded into a CUDA graph are not timed individually.
struct GemmProfile {
  bool on = false;
  std::vector<cudaEvent_t> ev;     // pairs (start, stop)
  std::vector<double> flops;       // per pair
  std::vector<int> phase;          // per pair: kPhGemm (FP64), kPhGemm32 (FP32) or kPhGemmTc
                                   // (FP64 as tensor-core digit-slice products)
};
extern thread_local GemmProfile g_gemm_prof;   // per calling thread (its context's profiler)

// Events around one launch of a kernel that has its own profiler phase (kPhK*); work is the
// launch's algorithmic work in that phase's unit. Inactive while profiling is off or the stream is
// being captured.
struct KernelTimer {
  cudaEvent_t e0 = nullptr;
  cudaStream_t s = nullptr;
  explicit KernelTimer(cudaStream_t st) : s(st) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap);
    if (g_gemm_prof.on && cap == cudaStreamCaptureStatusNone) {
      cudaEventCreate(&e0);
      cudaEventRecord(e0, s);
    }
  }
  void done(int phase, double work) {
    if (!e0) return;
    cudaEvent_t e1;
    cudaEventCreate(&e1);
    cudaEventRecord(e1, s);
    g_gemm_prof.ev.push_back(e0);
    g_gemm_prof.ev.push_back(e1);
    g_gemm_prof.flops.push_back(work);
    g_gemm_prof.phase.push_back(phase);
    e0 = nullptr;
  }
};

// In-place lower Cholesky A = L L^T (strict upper set to 0). status_dev[0] != 0 on failure.
void potrf_lower(cudaStream_t s, int n, double *A, int lda, int *status_dev);

// X = L^{-1} for lower-triangular L (X lower, strict upper zero), recursively on halves. work: >=
// n*n/4 doubles (more is used as split-K space).
void trtri_lower(cudaStream_t s, int n, const double *L, int ldl, double *X, int ldx, double *work,
                 size_t work_elems);

// Symmetric tridiagonal reduction A = Q T Q^T from the lower triangle of A (n x n, lda).
// d[n], e[n-1], tau[n-1]; V (n x n, ldv) receives the Householder vectors explicitly
// (column j: zeros for rows <= j, 1 at row j+1). work: sytrd_work_size<T>(n) elements. Each panel
// is one cooperative launch; if one of its bounded grid barriers gives up, *status (if given) is
// raised to kDevIterCap.
template <typename T>
size_t sytrd_work_size(int n);
template <typename T>
void sytrd_lower(cudaStream_t s, int n, T *A, int lda, T *d, T *e, T *tau, T *V, int ldv, T *work,
                 int *status = nullptr);

// Panel kernel of sytrd_lower (process-wide): 0 = tiles cut per column and re-read from memory for
// every column; 1 (default) = trailing tiles fixed per panel, resident in shared memory or streamed
// by TMA (sytrd_panel.cu) wherever the reduction fits its limits; 2 = as 1 with at most 64 CTAs and
// 8 tile slots, so that the streaming ring runs at small sizes (tests).
extern std::atomic<int> g_panel_mode;

struct GridBar;
// Launch plan of the resident-tile panel kernel for one reduction (A, n, lda fixed).
struct PanelResidentPlan {
  bool ok = false, tma = false;
  int nslot = 0, smem = 0, ctas = 0;
  alignas(64) unsigned char tmap[128];   // CUtensorMap of A (when tma)
};
template <typename T>
bool panel_resident_plan(int n, T *A, int lda, PanelResidentPlan &p);
// One panel (columns p0 .. p0 + nbp - 1) on `ctas` CTAs (at most p.ctas); the grid barrier counter
// stands at `base` when it starts and gains 2 nbp ctas arrivals.
template <typename T>
void panel_resident_launch(cudaStream_t s, const PanelResidentPlan &p, int ctas, T *A, int lda, int n, int p0, int nbp,
                           T *Vp, T *Wp, T *P, T *dots, T *part, T *vpart, T *dpart, T *V, int ldv, T *d, T *e,
                           T *tau, GridBar *bar, unsigned base, int *status);

// Z (n x k) <- Q Z with Q = H_0 ... H_{n-2} from sytrd_lower. work: ormtr_work_size<T>(n, k).
template <typename T>
size_t ormtr_work_size(int n, int k);
template <typename T>
void ormtr_left(cudaStream_t s, int n, int k, const T *V, int ldv, const T *tau, T *Z, int ldz, T *work);

// T (nb x nb, upper, leading dimension nb) of the compact WY form H_0 .. H_{nb-1} = I - V T V^T from
// G = V^T V (nb x nb) and tau[nb]; nb <= 64.
template <typename T>
void larft(cudaStream_t s, int nb, const T *G, const T *tau, T *Tf);

// Symmetric tridiagonal eigensolver (divide and conquer): d[n] (in: diagonal, out: eigenvalues
// ascending), e[n-1] off-diagonal (read only); Q (n x n, ldq = n) eigenvectors.
// work: stedc_work_size(n) elements of T, iwork: stedc_iwork_size(n) ints.
size_t stedc_work_size(int n);
size_t stedc_iwork_size(int n);
// Deflation of stedc's merges (process-wide): 1 (default) stages every merge that fits in shared
// memory (sequential scan at shared-memory latency, parallel compaction); 0 runs every merge's scan
// and compaction in global memory by one thread (the path merges above the staging limit take).
extern std::atomic<int> g_dc_stage;
template <typename T>
int stedc(cudaStream_t s, int n, T *d, T *e, T *Q, int ldq, T *work, int *iwork, int *status_dev);

// Small helpers
void set_zero(cudaStream_t s, double *p, size_t n);
template <typename T>
void set_zero_t(cudaStream_t s, T *p, size_t n);
template <typename T>
void copy_lower_to_upper(cudaStream_t s, int n, T *A, int lda);
void zero_strict_upper(cudaStream_t s, int n, double *A, int lda);
template <typename T>
void scale_columns(cudaStream_t s, int m, int n, const T *A, int lda, const double *f, T *B, int ldb);

}  // namespace dg
