// C-ABI of the dftbgpu library: context, model/geometry upload, the SCC driver and gradients.
// Host orchestration only; all numerical work runs in the kernels of linalg.cu, stedc.cu and
// dftb_kernels.cu on the context's stream.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <vector>

#include "batch.cuh"
#include "dftb_kernels.cuh"
#include "linalg.cuh"
#include "twostage.cuh"

namespace dg {

std::atomic<long long> g_launches{0};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  char err[1024] = {0};
  // model
  int nsp = 0;
  std::vector<SpeciesDev> h_sp;
  std::vector<PairDev> h_pair;
  SpeciesDev *d_sp = nullptr;
  PairDev *d_pair = nullptr;
  double *d_tab = nullptr;
  double *d_rep = nullptr;
  double sk_cut_max = 0.0;
  long long ham_len = 0;      // table values per kind (H or S), summed over ordered pairs
  bool have_model = false;
  // geometry
  int natom = 0, norb = 0;
  std::vector<int> h_species, h_orb_off;
  double *d_xyz = nullptr;
  int *d_species = nullptr;
  int *d_orb = nullptr;       // orb_off[natom+1] then orb_atom[norb]
  int *d_pcount = nullptr, *d_pstart = nullptr, *d_pi = nullptr, *d_pj = nullptr;
  int npairs = 0;
  size_t cap_atoms = 0, cap_pairs = 0;
  bool have_geom = false;
  // per-atom vectors
  double *d_q0 = nullptr, *d_qin = nullptr, *d_qout = nullptr, *d_V = nullptr, *d_Vout = nullptr,
         *d_eatom = nullptr, *d_grad = nullptr;
  std::vector<double> h_q0;
  // per-orbital vectors / matrices
  size_t cap_n = 0;
  double *H0 = nullptr, *S = nullptr, *Linv = nullptr, *H = nullptr, *T = nullptr, *Vh = nullptr,
         *Z = nullptr, *C = nullptr, *rho = nullptr, *W = nullptr;
  double *Lc = nullptr;   // Cholesky factor of S (lower)
  double *A0 = nullptr;   // L^-1 H0 L^-T (lower), per geometry (formed by the first SCC call)
  bool have_a0 = false;
  // FP32 eigensolver buffers of the mixed form (allocated on first use)
  size_t cap_n32 = 0;
  float *L32 = nullptr, *Li32 = nullptr, *A0_32 = nullptr, *A32 = nullptr, *T32 = nullptr, *V32 = nullptr,
        *Z32 = nullptr, *C32 = nullptr, *d32 = nullptr, *e32 = nullptr, *tau32 = nullptr, *wk32_sytrd = nullptr,
        *wk32_ormtr = nullptr, *wk32_stedc = nullptr, *wk32_ts = nullptr;
  double *wk_ts = nullptr;   // FP64 two-stage workspace (stage-level test hook)
  size_t cap_ts64 = 0;
  bool mixed_ready = false;
  int mixed_iters = 0;    // FP32 iterations of the last SCC call
  bool scc_mixed = false; // the last SCC call ran the mixed form
  // perturbative iterations of the mixed form: reference density and potentials of the last FP64
  // iteration, M^T / response matrix and C dP (n x n FP32); the FP32 LOW-iteration buffers hold
  // C (C32), X = S C (V32), diag(dV) C (T32), diag(dV) X (Z32) and drho (A32) meanwhile
  size_t cap_pert = 0, cap_pert_atoms = 0;
  float *Mt32 = nullptr, *Zp32 = nullptr;
  double *rho_ref = nullptr, *Vref = nullptr;
  // per-iteration record of the last SCC call: electronic energy, max|q_out - q_in|, precision, host ms
  std::vector<double> hist_e, hist_err, hist_ms;
  // batched form (many independent molecules sharing the model)
  BatchState *batch = nullptr;
  std::vector<int> hist_prec;
  double *eig = nullptr, *fill = nullptr, *fe = nullptr, *dd = nullptr, *ee = nullptr, *tau = nullptr,
         *qorb = nullptr, *eorb = nullptr;
  double *wk_sytrd = nullptr, *wk_ormtr = nullptr, *wk_stedc = nullptr;
  int *iwk_stedc = nullptr;
  int *d_status = nullptr;
  double *d_scal = nullptr;
  // Broyden
  int bro_cap_iter = 0;
  size_t bro_cap_atoms = 0;
  BroydenDev bro{};
  // SCC state
  bool have_scc = false;
  int nlevels = 0;
  bool have_w = false;
  double nel = 0.0;
  // phase timers (CUDA events on the stream)
  bool prof = false;
  std::vector<std::pair<int, cudaEvent_t>> marks;
  double prof_ms[kNPhase] = {0};
  double prof_flops[kNPhase] = {0};
  long long prof_calls[kNPhase] = {0};
};

// Record the start of a phase (phase < 0 closes the previous one).
static void mark(Ctx *c, int phase) {
  if (!c->prof) return;
  cudaEvent_t e;
  cudaEventCreate(&e);
  cudaEventRecord(e, c->stream);
  c->marks.push_back({phase, e});
}

static void prof_flops(Ctx *c, int phase, double f) {
  if (c->prof) c->prof_flops[phase] += f;
}

// Accumulate elapsed times between consecutive marks (called where the host synchronises anyway).
static void flush_marks(Ctx *c) {
  if (!c->prof) return;
  if (!c->marks.empty()) {
    cudaEventSynchronize(c->marks.back().second);
    for (size_t i = 0; i + 1 < c->marks.size(); ++i) {
      int ph = c->marks[i].first;
      if (ph < 0) continue;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c->marks[i].second, c->marks[i + 1].second);
      c->prof_ms[ph] += ms;
      c->prof_calls[ph] += 1;
    }
    for (size_t i = 0; i + 1 < c->marks.size(); ++i) cudaEventDestroy(c->marks[i].second);
    std::pair<int, cudaEvent_t> last = c->marks.back();
    c->marks.clear();
    if (last.first >= 0) c->marks.push_back(last);
    else cudaEventDestroy(last.second);
  }
  // GEMM and kernel-timer launches (also those of the stage test hooks, which set no marks)
  auto &gp = g_gemm_prof;
  for (size_t i = 0; i + 1 < gp.ev.size(); i += 2) {
    cudaEventSynchronize(gp.ev[i + 1]);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, gp.ev[i], gp.ev[i + 1]);
    const int ph = gp.phase[i / 2];
    c->prof_ms[ph] += ms;
    c->prof_flops[ph] += gp.flops[i / 2];
    c->prof_calls[ph] += 1;
    cudaEventDestroy(gp.ev[i]);
    cudaEventDestroy(gp.ev[i + 1]);
  }
  gp.ev.clear();
  gp.flops.clear();
  gp.phase.clear();
}

int set_error(Ctx *c, int code, const char *fmt, ...) {
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

template <class T>
static int dev_alloc(Ctx *c, T **p, size_t count) {
  if (*p) cudaFree(*p);
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void **)p, count * sizeof(T));
  if (e != cudaSuccess)
    return set_error(c, DFTBGPU_ERR_CUDA, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
  return DFTBGPU_OK;
}

// ------------------------------------------------------------------ host restatements (setup only)
static double host_neville8(const double *col, double incr, double x, int il) {
  double c[8], d[8], xp[8], delta[8];
  for (int ii = 0; ii < 8; ++ii) {
    xp[ii] = (double)(il - 8 + ii + 1) * incr;
    c[ii] = d[ii] = col[il - 8 + ii];
  }
  for (int mm = 1; mm < 8; ++mm) delta[mm] = 1.0 / (xp[mm] - xp[0]);
  int icl = (int)std::ceil((x - xp[0]) * delta[1]);
  double y = col[il - 8 + icl - 1];
  icl -= 1;
  for (int mm = 1; mm < 8; ++mm) {
    for (int i = 1; i <= 8 - mm; ++i) {
      double r2 = (d[i - 1] - c[i]) * delta[mm];
      c[i - 1] = (xp[i - 1] - x) * r2;
      d[i - 1] = (xp[i - 1 + mm] - x) * r2;
    }
    double dy;
    if (2 * icl < 8 - mm) dy = c[icl];
    else { dy = d[icl - 1]; icl -= 1; }
    y += dy;
  }
  return y;
}

static double host_gsub(double r, double t1, double t2) {
  double t12 = t1 * t1 - t2 * t2;
  return std::exp(-t1 * r) * ((0.5 * std::pow(t2, 4) * t1 / (t12 * t12)) -
                              (std::pow(t2, 6) - 3.0 * std::pow(t2, 4) * t1 * t1) / (r * t12 * t12 * t12));
}
static double host_exp_gamma(double r, double ua, double ub) {
  double ta = 3.2 * ua, tb = 3.2 * ub;
  if (r < 1e-5) {
    if (std::fabs(ua - ub) < 0.3125e-5) return -0.5 * (ua + ub);
    return -0.5 * ((ta * tb) / (ta + tb) + (ta * tb) * (ta * tb) / std::pow(ta + tb, 3));
  }
  if (std::fabs(ua - ub) < 0.3125e-5) {
    double tm = 0.5 * (ta + tb);
    return std::exp(-tm * r) * (1.0 / r + 0.6875 * tm + 0.1875 * r * tm * tm +
                                0.02083333333333333333 * r * r * tm * tm * tm);
  }
  return host_gsub(r, ta, tb) + host_gsub(r, tb, ta);
}
// shortgammafuncs.F90:27-94 (expGammaCutoff): distance where the short gamma drops below 1e-10.
static double host_gamma_cutoff(double u2, double u1) {
  const double cv = 1e-10, tol = 1e-10;
  double rab = 1.0;
  while (host_exp_gamma(rab, u2, u1) > cv) rab *= 2.0;
  double min_cut = rab + 0.1, max_cut = 0.5 * rab - 0.1;
  double max_g = host_exp_gamma(max_cut, u2, u1), min_g = host_exp_gamma(min_cut, u2, u1);
  double lower_g = host_exp_gamma(min_cut, u2, u1);
  double cut = max_cut + 0.1;
  double g = host_exp_gamma(cut, u2, u1);
  int guard = 0;
  while ((g - lower_g) > tol && guard++ < 10000) {
    max_cut = 0.5 * (cut + min_cut);
    if ((max_g >= min_g) == (cv >= host_exp_gamma(max_cut, u2, u1))) {
      min_cut = max_cut;
      lower_g = host_exp_gamma(min_cut, u2, u1);
    } else {
      cut = max_cut;
      g = host_exp_gamma(cut, u2, u1);
    }
  }
  return min_cut;
}

// ------------------------------------------------------------------ buffers
static int ensure_atoms(Ctx *c, int natom) {
  if ((size_t)natom <= c->cap_atoms) return DFTBGPU_OK;
  size_t n = natom;
  DG_CHECK(c, dev_alloc(c, &c->d_xyz, 3 * n));
  DG_CHECK(c, dev_alloc(c, &c->d_species, n));
  DG_CHECK(c, dev_alloc(c, &c->d_pcount, n));
  DG_CHECK(c, dev_alloc(c, &c->d_pstart, n + 1));
  DG_CHECK(c, dev_alloc(c, &c->d_q0, n));
  DG_CHECK(c, dev_alloc(c, &c->d_qin, n));
  DG_CHECK(c, dev_alloc(c, &c->d_qout, n));
  DG_CHECK(c, dev_alloc(c, &c->d_V, n));
  DG_CHECK(c, dev_alloc(c, &c->d_Vout, n));
  DG_CHECK(c, dev_alloc(c, &c->d_eatom, n));
  DG_CHECK(c, dev_alloc(c, &c->d_grad, 3 * n));
  c->cap_atoms = n;
  return DFTBGPU_OK;
}

static int ensure_orbitals(Ctx *c, int n) {
  if ((size_t)n <= c->cap_n) return DFTBGPU_OK;
  size_t nn = (size_t)n * n;
  for (double **p : {&c->H0, &c->S, &c->Linv, &c->H, &c->T, &c->Vh, &c->Z, &c->C, &c->rho, &c->W, &c->Lc,
                     &c->A0})
    DG_CHECK(c, dev_alloc(c, p, nn));
  for (double **p : {&c->eig, &c->fill, &c->fe, &c->dd, &c->ee, &c->tau, &c->qorb, &c->eorb})
    DG_CHECK(c, dev_alloc(c, p, (size_t)n));
  DG_CHECK(c, dev_alloc(c, &c->wk_sytrd, sytrd_work_size<double>(n)));
  DG_CHECK(c, dev_alloc(c, &c->wk_ormtr, ormtr_work_size<double>(n, n)));
  DG_CHECK(c, dev_alloc(c, &c->wk_stedc, stedc_work_size(n)));
  DG_CHECK(c, dev_alloc(c, &c->iwk_stedc, stedc_iwork_size(n)));
  c->cap_n = n;
  return DFTBGPU_OK;
}

static int ensure_broyden(Ctx *c, int natom, int max_iter) {
  if (c->bro_cap_iter >= max_iter && c->bro_cap_atoms >= (size_t)natom) return DFTBGPU_OK;
  int M = max_iter;
  size_t N = natom;
  DG_CHECK(c, dev_alloc(c, &c->bro.ww, M));
  DG_CHECK(c, dev_alloc(c, &c->bro.aa, (size_t)M * M));
  DG_CHECK(c, dev_alloc(c, &c->bro.dF, N * M));
  DG_CHECK(c, dev_alloc(c, &c->bro.uu, N * M));
  DG_CHECK(c, dev_alloc(c, &c->bro.qlast, N));
  DG_CHECK(c, dev_alloc(c, &c->bro.dlast, N));
  c->bro.max_iter = M;
  c->bro_cap_iter = M;
  c->bro_cap_atoms = N;
  return DFTBGPU_OK;
}

// FP32 buffers of the reduced-precision eigensolves.
static int ensure_mixed_buffers(Ctx *c, int n) {
  if ((size_t)n > c->cap_n32) {
    size_t nn = (size_t)n * n;
    for (float **p : {&c->L32, &c->Li32, &c->A0_32, &c->A32, &c->T32, &c->V32, &c->Z32, &c->C32})
      DG_CHECK(c, dev_alloc(c, p, nn));
    for (float **p : {&c->d32, &c->e32, &c->tau32}) DG_CHECK(c, dev_alloc(c, p, (size_t)n));
    DG_CHECK(c, dev_alloc(c, &c->wk32_sytrd, sytrd_work_size<float>(n)));
    DG_CHECK(c, dev_alloc(c, &c->wk32_ormtr, ormtr_work_size<float>(n, n)));
    DG_CHECK(c, dev_alloc(c, &c->wk32_stedc, stedc_work_size(n)));
    DG_CHECK(c, dev_alloc(c, &c->wk32_ts, twostage_work_size<float>(n)));
    c->cap_n32 = n;
    c->mixed_ready = false;
  }
  return DFTBGPU_OK;
}

// FP32 copies of L, L^-1 and A0 for the reduced-precision iterations (once per geometry).
static int ensure_mixed(Ctx *c, int n) {
  DG_CHECK(c, ensure_mixed_buffers(c, n));
  // size the tensor-core FP64 scratch once; if the device cannot hold it, the FP64 products of the
  // mixed form stay on FP64 FMA (gemm<double> falls back per product)
  if (g_tc_dgemm_mixed) tc_dgemm_reserve(n, n, n);
  if (!c->mixed_ready) {
    size_t nn = (size_t)n * n;
    convert_d2f(c->stream, nn, c->Lc, c->L32);
    convert_d2f(c->stream, nn, c->Linv, c->Li32);
    convert_d2f(c->stream, nn, c->A0, c->A0_32);
    c->mixed_ready = true;
  }
  return DFTBGPU_OK;
}

static int ensure_pert(Ctx *c, int n, int natom) {
  if ((size_t)n > c->cap_pert) {
    size_t nn = (size_t)n * n;
    DG_CHECK(c, dev_alloc(c, &c->Mt32, nn));
    DG_CHECK(c, dev_alloc(c, &c->Zp32, nn));
    DG_CHECK(c, dev_alloc(c, &c->rho_ref, nn));
    c->cap_pert = n;
  }
  if ((size_t)natom > c->cap_pert_atoms) {
    DG_CHECK(c, dev_alloc(c, &c->Vref, (size_t)natom));
    c->cap_pert_atoms = natom;
  }
  return DFTBGPU_OK;
}

template <typename T>
__global__ void identity_kernel(int n, T *Z) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) Z[i + i * (long long)n] = T(1);
}
static void identity_f(cudaStream_t s, int n, float *Z) {
  identity_kernel<float><<<ceil_div(n, 256), 256, 0, s>>>(n, Z);
  count_launch();
}
static void identity_d(cudaStream_t s, int n, double *Z) {
  identity_kernel<double><<<ceil_div(n, 256), 256, 0, s>>>(n, Z);
  count_launch();
}

static ModelDev model_view(Ctx *c) { return ModelDev{c->nsp, c->d_sp, c->d_pair, c->d_tab, c->d_rep}; }
static GeomDev geom_view(Ctx *c) { return GeomDev{c->natom, c->norb, c->d_xyz, c->d_species, c->d_orb}; }

static int check_status(Ctx *c, const char *stage) {
  int st = 0;
  DG_CUDA(c, cudaMemcpyAsync(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  DG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (st == kDevNotPosDef) return set_error(c, DFTBGPU_ERR_NOT_POSDEF, "%s: overlap matrix is not positive definite", stage);
  if (st == kDevIterCap) return set_error(c, DFTBGPU_ERR_ITER_CAP, "%s: secular equation iteration cap reached", stage);
  if (st != 0) return set_error(c, DFTBGPU_ERR_CUDA, "%s: device status %d", stage, st);
  return DFTBGPU_OK;
}

// Generalized eigensolve of H (full symmetric, destroyed) with the stored L^-1. Eigenvalues into
// c->eig; the eigenvectors of the first k levels into c->C (columns), k chosen by pick_k after the
// eigenvalues are known (the Fermi filling decides how many levels the density matrix needs).
// all_vectors: back-transform all n eigenvectors (c->Z = Y, c->C = L^-T Y), k is still returned.
template <class PickK>
static int eigensolve(Ctx *c, int n, double *Hm, PickK pick_k, bool reduced = false, bool all_vectors = false) {
  cudaStream_t s = c->stream;
  const double nd = (double)n;
  if (!reduced) {
    // A = L^-1 H L^-T : T = H L^-T (L^-T upper), A(lower) = L^-1 T (L^-1 lower)
    mark(c, kPhTransform);
    prof_flops(c, kPhTransform, nd * nd * nd);
    dgemm(s, 'N', 'T', n, n, n, 1.0, Hm, n, c->Linv, n, 0.0, c->T, n, kBUpper);
    dgemm(s, 'N', 'N', n, n, n, 1.0, c->Linv, n, c->T, n, 0.0, Hm, n, kALower | kCLower);
  }
  mark(c, kPhSytrd);
  prof_flops(c, kPhSytrd, 4.0 / 3.0 * nd * nd * nd);
  sytrd_lower(s, n, Hm, n, c->dd, c->ee, c->tau, c->Vh, n, c->wk_sytrd, c->d_status);
  mark(c, kPhStedc);
  int rc = stedc(s, n, c->dd, c->ee, c->Z, n, c->wk_stedc, c->iwk_stedc, c->d_status);
  if (rc != 0) return set_error(c, DFTBGPU_ERR_ARGS, "stedc workspace layout error");
  DG_CUDA(c, cudaMemcpyAsync(c->eig, c->dd, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  mark(c, kPhFermi);
  int k = 0;
  DG_CHECK(c, pick_k(&k));
  mark(c, kPhBack);
  const int kb = all_vectors ? n : k;
  if (kb > 0) {
    prof_flops(c, kPhBack, 3.0 * nd * nd * (double)kb);
    ormtr_left(s, n, kb, c->Vh, n, c->tau, c->Z, n, c->wk_ormtr);
    dgemm(s, 'T', 'N', n, kb, n, 1.0, c->Linv, n, c->Z, n, 0.0, c->C, n, kAUpper);
  }
  return DFTBGPU_OK;
}

// L^-1 and the reduced non-SCC Hamiltonian A0 = L^-1 H0 L^-T (lower), once per geometry, formed by
// the first SCC call so that the mixed form can run their products on the tensor cores (g_tc_dgemm
// set by the caller); the plain form forms them in FP64 arithmetic. (The Cholesky factor itself is
// computed by set_geometry, which reports an overlap that is not positive definite.)
static int ensure_a0(Ctx *c) {
  if (c->have_a0) return DFTBGPU_OK;
  cudaStream_t s = c->stream;
  const int n = c->norb;
  mark(c, kPhH0S);
  prof_flops(c, kPhH0S, (double)n * n * n);
  trtri_lower(s, n, c->Lc, n, c->Linv, n, c->T, (size_t)n * n);
  dgemm(s, 'N', 'T', n, n, n, 1.0, c->H0, n, c->Linv, n, 0.0, c->T, n, kBUpper);
  dgemm(s, 'N', 'N', n, n, n, 1.0, c->Linv, n, c->T, n, 0.0, c->A0, n, kALower | kCLower);
  c->have_a0 = true;
  return DFTBGPU_OK;
}

static int density(Ctx *c, int n, int k, const double *w, double *out) {
  cudaStream_t s = c->stream;
  if (k <= 0) {
    set_zero(s, out, (size_t)n * n);
    return DFTBGPU_OK;
  }
  scale_columns(s, n, k, c->C, n, w, c->T, n);
  dgemm(s, 'N', 'T', n, n, k, 1.0, c->T, n, c->C, n, 0.0, out, n, kCLower);
  copy_lower_to_upper(s, n, out, n);
  return DFTBGPU_OK;
}

}  // namespace dg

using namespace dg;

struct dftbgpu_ctx : public dg::Ctx {};

extern "C" {

void dftbgpu_default_opts(dftbgpu_scc_opts *o) {
  if (!o) return;
  o->kT = 0.0;
  o->scc_tol = 1e-5;
  o->max_iter = 100;
  o->min_iter = 1;
  o->mix_alpha = 0.2;
  o->mix_omega0 = 0.01;
  o->mix_min_weight = 1.0;
  o->mix_max_weight = 1e5;
  o->mix_weight_fac = 1e-2;
  o->net_charge = 0.0;
  o->precision = DFTBGPU_PREC_FP64;
  o->convergent_only = 0;
  o->mixed_switch_tol = 0.0;
}

int dftbgpu_create(dftbgpu_ctx **out, int device) {
  if (!out) return DFTBGPU_ERR_ARGS;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return DFTBGPU_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return DFTBGPU_ERR_ARGS;
  dftbgpu_ctx *c = new dftbgpu_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return DFTBGPU_ERR_CUDA;
  }
  if (dev_alloc(c, &c->d_status, 4) || dev_alloc(c, &c->d_scal, kSCount)) {
    delete c;
    return DFTBGPU_ERR_CUDA;
  }
  cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream);
  *out = c;
  return DFTBGPU_OK;
}

int dftbgpu_destroy(dftbgpu_ctx *c) {
  if (!c) return DFTBGPU_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  void *ptrs[] = {c->d_sp, c->d_pair, c->d_tab, c->d_rep, c->d_xyz, c->d_species, c->d_orb, c->d_pcount,
                  c->d_pstart, c->d_pi, c->d_pj, c->d_q0, c->d_qin, c->d_qout, c->d_V, c->d_Vout,
                  c->d_eatom, c->d_grad, c->H0, c->S, c->Linv, c->H, c->T, c->Vh, c->Z, c->C, c->rho,
                  c->W, c->Lc, c->A0, c->eig, c->fill, c->fe, c->dd, c->ee, c->tau, c->qorb, c->eorb, c->wk_sytrd,
                  c->wk_ormtr, c->wk_stedc, c->iwk_stedc, c->d_status, c->d_scal, c->bro.ww, c->bro.aa,
                  c->bro.dF, c->bro.uu, c->bro.qlast, c->bro.dlast, c->L32, c->Li32, c->A0_32, c->A32,
                  c->T32, c->V32, c->Z32, c->C32, c->d32, c->e32, c->tau32, c->wk32_sytrd, c->wk32_ormtr,
                  c->wk32_stedc, c->Mt32, c->Zp32, c->rho_ref, c->Vref, c->wk32_ts, c->wk_ts};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (c->batch) {
    batch_free(*c->batch);
    delete c->batch;
  }
  cudaStreamDestroy(c->stream);
  delete c;
  return DFTBGPU_OK;
}

const char *dftbgpu_last_error(const dftbgpu_ctx *c) { return c ? c->err : "null context"; }

long long dftbgpu_kernel_launches(const dftbgpu_ctx *) { return dg::g_launches; }

int dftbgpu_set_model(dftbgpu_ctx *c, int nsp, const int *n_shell, const int *ang_shell, const double *onsite,
                      const double *hubbu, const double *ref_occ, const double *sk_dist, const int *sk_rows,
                      const int *sk_nint, const double *sk_ham, const double *sk_over, const int *rep_nspline,
                      const double *rep_data) {
  if (!c) return DFTBGPU_ERR_ARGS;
  if (nsp <= 0 || !n_shell || !ang_shell || !onsite || !hubbu || !ref_occ || !sk_dist || !sk_rows || !sk_nint ||
      !sk_ham || !sk_over || !rep_nspline || !rep_data)
    return set_error(c, DFTBGPU_ERR_ARGS, "set_model: null argument or nsp <= 0");
  cudaSetDevice(c->device);
  c->nsp = nsp;
  c->h_sp.assign(nsp, SpeciesDev{});
  for (int a = 0; a < nsp; ++a) {
    SpeciesDev &sp = c->h_sp[a];
    sp.n_shell = n_shell[a];
    if (sp.n_shell < 1 || sp.n_shell > kMaxShell)
      return set_error(c, DFTBGPU_ERR_ARGS, "species %d: %d shells (1..%d supported)", a, sp.n_shell, kMaxShell);
    sp.n_orb = 0;
    for (int k = 0; k < kMaxShell; ++k) {
      sp.ang[k] = (k < sp.n_shell) ? ang_shell[a * kMaxShell + k] : -1;
      sp.onsite[k] = onsite[a * kMaxShell + k];
      sp.occ[k] = ref_occ[a * kMaxShell + k];
      if (k < sp.n_shell) {
        if (sp.ang[k] < 0 || sp.ang[k] > 2)
          return set_error(c, DFTBGPU_ERR_ARGS, "species %d shell %d: l=%d (s, p, d supported)", a, k, sp.ang[k]);
        sp.n_orb += 2 * sp.ang[k] + 1;
      }
    }
    if (sp.n_orb > kMaxOrb) return set_error(c, DFTBGPU_ERR_ARGS, "species %d: %d orbitals > %d", a, sp.n_orb, kMaxOrb);
    sp.hubbu = hubbu[a];
    if (!(sp.hubbu > 1e-6)) return set_error(c, DFTBGPU_ERR_ARGS, "species %d: Hubbard U too small", a);
  }
  c->h_pair.assign((size_t)nsp * nsp, PairDev{});
  long long off = 0, roff = 0;
  long long ham_off = 0;
  for (int p = 0; p < nsp * nsp; ++p) ham_off += (long long)sk_rows[p] * sk_nint[p];
  c->ham_len = ham_off;
  std::vector<double> tab(2 * (size_t)ham_off);
  std::memcpy(tab.data(), sk_ham, sizeof(double) * ham_off);
  std::memcpy(tab.data() + ham_off, sk_over, sizeof(double) * ham_off);
  long long rep_total = 0;
  for (int p = 0; p < nsp * nsp; ++p) rep_total += 4 + rep_nspline[p] + 4LL * (rep_nspline[p] - 1) + 6;
  c->sk_cut_max = 0.0;
  for (int a = 0; a < nsp; ++a)
    for (int b = 0; b < nsp; ++b) {
      int p = a * nsp + b;
      PairDev &P = c->h_pair[p];
      P.dist = sk_dist[p];
      P.rows = sk_rows[p];
      P.n_int = sk_nint[p];
      int want = 0;
      for (int i = 0; i < c->h_sp[a].n_shell; ++i)
        for (int j = 0; j < c->h_sp[b].n_shell; ++j) want += std::min(c->h_sp[a].ang[i], c->h_sp[b].ang[j]) + 1;
      if (P.n_int != want || P.n_int > kMaxInt)
        return set_error(c, DFTBGPU_ERR_ARGS, "pair %d-%d: %d integrals, expected %d", a, b, P.n_int, want);
      if (P.rows < 9 || !(P.dist > 0))
        return set_error(c, DFTBGPU_ERR_ARGS, "pair %d-%d: not enough points in the SK table", a, b);
      P.off_ham = off;
      P.off_over = ham_off + off;
      P.sk_cut = P.rows * P.dist + 1.0;
      c->sk_cut_max = std::max(c->sk_cut_max, P.sk_cut);
      // 5th-order tail coefficients (slakoeqgrid.F90:225-241), per integral
      for (int k = 0; k < P.n_int; ++k) {
        for (int m = 0; m < 2; ++m) {
          const double *col = tab.data() + (m ? P.off_over : P.off_ham) + (size_t)k * P.rows;
          double xa8 = (double)P.rows * P.dist;
          double y0 = host_neville8(col, P.dist, xa8 - 1e-5, P.rows);
          double y2 = host_neville8(col, P.dist, xa8 + 1e-5, P.rows);
          double y1 = col[P.rows - 1];
          double (*tl)[kMaxInt] = m ? P.tail_s : P.tail_h;
          tl[0][k] = y1;
          tl[1][k] = (y2 - y0) / (2.0 * 1e-5);
          tl[2][k] = (y2 + y0 - 2.0 * y1) / (1e-5 * 1e-5);
        }
      }
      off += (long long)P.rows * P.n_int;
      P.off_rep = roff;
      P.n_spline = rep_nspline[p];
      P.rep_cut = rep_data[roff];
      roff += 4 + P.n_spline + 4LL * (P.n_spline - 1) + 6;
      P.gamma_cut = host_gamma_cutoff(c->h_sp[b].hubbu, c->h_sp[a].hubbu);
    }
  DG_CHECK(c, dev_alloc(c, &c->d_sp, (size_t)nsp));
  DG_CHECK(c, dev_alloc(c, &c->d_pair, (size_t)nsp * nsp));
  DG_CHECK(c, dev_alloc(c, &c->d_tab, tab.size()));
  DG_CHECK(c, dev_alloc(c, &c->d_rep, (size_t)rep_total));
  DG_CUDA(c, cudaMemcpyAsync(c->d_sp, c->h_sp.data(), sizeof(SpeciesDev) * nsp, cudaMemcpyHostToDevice, c->stream));
  DG_CUDA(c, cudaMemcpyAsync(c->d_pair, c->h_pair.data(), sizeof(PairDev) * nsp * nsp, cudaMemcpyHostToDevice, c->stream));
  DG_CUDA(c, cudaMemcpyAsync(c->d_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, c->stream));
  DG_CUDA(c, cudaMemcpyAsync(c->d_rep, rep_data, sizeof(double) * rep_total, cudaMemcpyHostToDevice, c->stream));
  DG_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_model = true;
  c->have_geom = false;
  c->have_scc = false;
  return DFTBGPU_OK;
}

// host_pi / host_pj: a half pair list (i < j, sorted) given by the caller instead of the GPU's own
static int set_geometry_impl(dftbgpu_ctx *c, int natom, const double *coords, bool dev, const int *species,
                             const std::vector<int> *host_pi = nullptr, const std::vector<int> *host_pj = nullptr) {
  if (!c) return DFTBGPU_ERR_ARGS;
  if (!c->have_model) return set_error(c, DFTBGPU_ERR_STATE, "set_geometry: no model set");
  if (natom <= 0 || !coords || !species) return set_error(c, DFTBGPU_ERR_ARGS, "set_geometry: bad arguments");
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  c->h_species.assign(species, species + natom);
  c->h_orb_off.assign(natom + 1, 0);
  c->h_q0.assign(natom, 0.0);
  for (int a = 0; a < natom; ++a) {
    int sp = species[a];
    if (sp < 0 || sp >= c->nsp) return set_error(c, DFTBGPU_ERR_ARGS, "atom %d: species %d out of range", a, sp);
    c->h_orb_off[a + 1] = c->h_orb_off[a] + c->h_sp[sp].n_orb;
    double q = 0.0;
    for (int k = 0; k < c->h_sp[sp].n_shell; ++k) q += c->h_sp[sp].occ[k];
    c->h_q0[a] = q;
  }
  int norb = c->h_orb_off[natom];
  DG_CHECK(c, ensure_atoms(c, natom));
  DG_CHECK(c, ensure_orbitals(c, norb));
  DG_CHECK(c, dev_alloc(c, &c->d_orb, (size_t)natom + 1 + norb));
  std::vector<int> orb(natom + 1 + norb);
  for (int a = 0; a <= natom; ++a) orb[a] = c->h_orb_off[a];
  for (int a = 0; a < natom; ++a)
    for (int o = c->h_orb_off[a]; o < c->h_orb_off[a + 1]; ++o) orb[natom + 1 + o] = a;
  c->natom = natom;
  c->norb = norb;
  DG_CUDA(c, cudaMemcpyAsync(c->d_orb, orb.data(), sizeof(int) * orb.size(), cudaMemcpyHostToDevice, s));
  DG_CUDA(c, cudaMemcpyAsync(c->d_species, species, sizeof(int) * natom, cudaMemcpyHostToDevice, s));
  DG_CUDA(c, cudaMemcpyAsync(c->d_xyz, coords, sizeof(double) * 3 * natom,
                             dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  DG_CUDA(c, cudaMemcpyAsync(c->d_q0, c->h_q0.data(), sizeof(double) * natom, cudaMemcpyHostToDevice, s));
  DG_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
  GeomDev g = geom_view(c);
  ModelDev m = model_view(c);
  // neighbour list (pairs within the SK cutoff); the pair arrays grow on demand
  int np = 0;
  if (host_pi) {
    np = (int)host_pi->size();
    if (c->cap_pairs < (size_t)np || !c->d_pi) {
      DG_CHECK(c, dev_alloc(c, &c->d_pi, (size_t)std::max(np, 1)));
      DG_CHECK(c, dev_alloc(c, &c->d_pj, (size_t)std::max(np, 1)));
      c->cap_pairs = (size_t)std::max(np, 1);
    }
    if (np > 0) {
      DG_CUDA(c, cudaMemcpyAsync(c->d_pi, host_pi->data(), sizeof(int) * np, cudaMemcpyHostToDevice, s));
      DG_CUDA(c, cudaMemcpyAsync(c->d_pj, host_pj->data(), sizeof(int) * np, cudaMemcpyHostToDevice, s));
    }
  } else {
    // count first to size the arrays
    size_t need = (size_t)natom * 64;
    if (c->cap_pairs < need) {
      DG_CHECK(c, dev_alloc(c, &c->d_pi, need));
      DG_CHECK(c, dev_alloc(c, &c->d_pj, need));
      c->cap_pairs = need;
    }
    build_pairs(s, g, c->sk_cut_max, c->d_pcount, c->d_pstart, c->d_pi, c->d_pj, c->cap_pairs, &np);
    if ((size_t)np > c->cap_pairs) {
      DG_CHECK(c, dev_alloc(c, &c->d_pi, (size_t)np));
      DG_CHECK(c, dev_alloc(c, &c->d_pj, (size_t)np));
      c->cap_pairs = np;
      build_pairs(s, g, c->sk_cut_max, c->d_pcount, c->d_pstart, c->d_pi, c->d_pj, c->cap_pairs, &np);
    }
  }
  c->npairs = np;
  mark(c, kPhH0S);
  prof_flops(c, kPhH0S, (double)norb * norb * norb / 3.0);
  build_h0_s(s, m, g, c->d_pi, c->d_pj, np, c->H0, c->S);
  repulsive_energy(s, m, g, c->d_eatom, c->d_scal);
  // Cholesky of S (L^-1 and A0 = L^-1 H0 L^-T follow in the first SCC call: ensure_a0)
  DG_CUDA(c, cudaMemcpyAsync(c->Lc, c->S, sizeof(double) * (size_t)norb * norb, cudaMemcpyDeviceToDevice, s));
  potrf_lower(s, norb, c->Lc, norb, c->d_status);
  DG_CHECK(c, check_status(c, "Cholesky of S"));
  mark(c, -1);
  DG_CUDA(c, cudaGetLastError());
  DG_CUDA(c, cudaStreamSynchronize(s));
  flush_marks(c);
  c->have_geom = true;
  c->have_scc = false;
  c->have_w = false;
  c->mixed_ready = false;
  c->have_a0 = false;
  return DFTBGPU_OK;
}

int dftbgpu_set_geometry(dftbgpu_ctx *c, int natom, const double *coords, const int *species) {
  return set_geometry_impl(c, natom, coords, false, species);
}

int dftbgpu_set_geometry_dev(dftbgpu_ctx *c, int natom, const double *coords_dev, const int *species_host) {
  return set_geometry_impl(c, natom, coords_dev, true, species_host);
}

int dftbgpu_set_geometry_neighbours(dftbgpu_ctx *c, int natom, const double *coords, const int *species,
                                    const int *nneigh, const int *ineigh, int maxneigh) {
  if (!c) return DFTBGPU_ERR_ARGS;
  if (natom <= 0 || !coords || !species || !nneigh || !ineigh || maxneigh < 0)
    return set_error(c, DFTBGPU_ERR_ARGS, "set_geometry_neighbours: bad arguments");
  // each pair once as (min, max), sorted like the GPU's own list
  std::vector<long long> keys;
  for (int i = 0; i < natom; ++i) {
    if (nneigh[i] < 0 || nneigh[i] > maxneigh)
      return set_error(c, DFTBGPU_ERR_ARGS, "set_geometry_neighbours: atom %d has %d neighbours (max %d)", i,
                       nneigh[i], maxneigh);
    const int *row = ineigh + (size_t)i * (maxneigh + 1);
    for (int k = 1; k <= nneigh[i]; ++k) {
      const int j = row[k];
      if (j < 0 || j >= natom)
        return set_error(c, DFTBGPU_ERR_ARGS,
                         "set_geometry_neighbours: neighbour %d of atom %d is not an atom of the cluster", j, i);
      if (j == i) continue;
      keys.push_back((long long)std::min(i, j) * natom + std::max(i, j));
    }
  }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  std::vector<int> pi(keys.size()), pj(keys.size());
  for (size_t p = 0; p < keys.size(); ++p) {
    pi[p] = (int)(keys[p] / natom);
    pj[p] = (int)(keys[p] % natom);
  }
  return set_geometry_impl(c, natom, coords, false, species, &pi, &pj);
}

int dftbgpu_scc(dftbgpu_ctx *c, const dftbgpu_scc_opts *o, const double *q_init, dftbgpu_energies *energies,
                double *ef, double *eigen, double *filling, double *q_out, int *n_iter, int *converged) {
  if (!c || !o) return DFTBGPU_ERR_ARGS;
  if (!c->have_geom) return set_error(c, DFTBGPU_ERR_STATE, "scc: no geometry set");
  if (o->max_iter < 1 || o->max_iter > 150) return set_error(c, DFTBGPU_ERR_ARGS, "scc: max_iter must be in 1..150");
  if (!(o->kT > 0.0)) return set_error(c, DFTBGPU_ERR_ARGS, "scc: kT must be > 0 (Fermi filling)");
  if (o->precision != DFTBGPU_PREC_FP64 && o->precision != DFTBGPU_PREC_MIXED)
    return set_error(c, DFTBGPU_ERR_ARGS, "scc: unknown precision form %d", o->precision);
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int n = c->norb, N = c->natom;
  GeomDev g = geom_view(c);
  ModelDev m = model_view(c);
  DG_CHECK(c, ensure_broyden(c, N, o->max_iter));
  double nel = 0.0;
  for (double q : c->h_q0) nel += q;
  nel -= o->net_charge;
  c->nel = nel;
  if (q_init) DG_CUDA(c, cudaMemcpyAsync(c->d_qin, q_init, sizeof(double) * N, cudaMemcpyHostToDevice, s));
  else DG_CUDA(c, cudaMemcpyAsync(c->d_qin, c->d_q0, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
  DG_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
  double h_scal[kSCount];
  int it = 0;
  bool conv = false;
  // Mixed form, three kinds of iteration:
  //   LOW  FP32 eigensolve (transform, tridiagonalisation, divide and conquer, back-transform,
  //        density) until max|q_out - q_in| < switch_tol;
  //   FULL FP64 eigensolve with all eigenvectors, which becomes the reference of
  //   PERT first-order density-matrix perturbation around the last FULL iteration (FP32 GEMMs on
  //        the potential change only), until converged; then FULL again at the same charges.
  // The cycle only ends on a converged FULL iteration, so every returned state is FP64. The plain
  // form runs FULL iterations (with k eigenvectors) throughout.
  enum { kFormLow, kFormFull, kFormPert };
  const bool mixed = (o->precision == DFTBGPU_PREC_MIXED);
  int form = mixed ? kFormLow : kFormFull;
  const double switch_tol = (o->mixed_switch_tol > 0.0) ? o->mixed_switch_tol : 3e-3;
  constexpr int kMaxPertRun = 16;   // perturbative iterations before the reference is renewed
  int pert_run = 0, k_ref = 0;
  bool verify = false;   // the next FULL iteration checks a converged perturbative state (k vectors)
  g_tc_dgemm = mixed && g_tc_dgemm_mixed;
  DG_CHECK(c, ensure_a0(c));
  g_tc_dgemm = false;
  if (mixed) {
    DG_CHECK(c, ensure_mixed(c, n));
    DG_CHECK(c, ensure_pert(c, n, N));
  }
  c->mixed_iters = 0;
  c->scc_mixed = mixed;
  // gemm<double> goes to the tensor-core digit-slice product only inside the mixed form's FP64
  // iterations; the guard switches it off again on every return path
  struct RouteGuard {
    ~RouteGuard() {
      g_tc_dgemm = false;
      g_tc_fgemm = false;
    }
  } route_guard;
  c->hist_e.clear(); c->hist_err.clear(); c->hist_ms.clear(); c->hist_prec.clear();
  int mix_calls = 0;
  auto pick = [&](int *kout) -> int {
    fermi_filling(s, n, c->eig, nel, o->kT, c->fill, c->d_scal);
    DG_CUDA(c, cudaMemcpyAsync(h_scal, c->d_scal, sizeof(h_scal), cudaMemcpyDeviceToHost, s));
    DG_CUDA(c, cudaStreamSynchronize(s));
    int st = 0;
    DG_CUDA(c, cudaMemcpy(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st == kDevIterCap) return set_error(c, DFTBGPU_ERR_ITER_CAP, "eigensolver: a bounded device loop hit its cap (secular iteration or grid barrier)");
    if (h_scal[kSFermiStatus] != 0.0) return set_error(c, DFTBGPU_ERR_FERMI, "Fermi level search did not converge.");
    *kout = (int)h_scal[kSNLevels];
    return DFTBGPU_OK;
  };
  for (it = 1; it <= o->max_iter; ++it) {
    const auto t_it = std::chrono::steady_clock::now();
    if (mixed && it == o->max_iter) form = kFormFull;   // the last allowed iteration is FP64
    const int it_form = form;
    g_tc_dgemm = mixed && g_tc_dgemm_mixed && form == kFormFull;
    g_tc_fgemm = mixed && g_tc_fgemm_mixed;   // FP32 products of the FP32 eigensolves and the reference
    mark(c, kPhPot);
    potential(s, m, g, c->d_qin, c->d_q0, c->d_V);
    int k = 0;
    if (form == kFormPert) {
      // rho = rho_ref + C dP C^T with dP from M = C^T dH C, dH = 1/2 (S D + D S), D = diag(V - Vref)
      mark(c, kPhPert);
      const double nd = (double)n;
      k = k_ref;
      prof_flops(c, kPhPert, 8.0 * nd * nd * (double)k);
      dmpt_scale(s, g, c->d_V, c->Vref, c->C32, c->V32, c->T32, c->Z32);
      // FP32 products: tcgen05 split-BF16 tensor cores, or FP32 FMA when they are switched off
      auto pgemm = [&](char ta, char tb, int mm, int nn, int kk, float al, const float *A, const float *B, float be,
                       float *Cc, int fl) {
        if (g_tc_gemm && mm >= 128 && nn >= 128) return tc_gemm(s, ta, tb, mm, nn, kk, al, A, n, B, n, be, Cc, n, fl);
        gemm<float>(s, ta, tb, mm, nn, kk, al, A, n, B, n, be, Cc, n, fl);
        return 0;
      };
      int grc = 0;
      grc |= pgemm('T', 'N', n, k, n, 0.5f, c->T32, c->V32, 0.f, c->Mt32, 0);
      grc |= pgemm('T', 'N', n, k, n, 0.5f, c->Z32, c->C32, 1.f, c->Mt32, 0);
      dmpt_dmu(s, n, k, c->Mt32, c->fill, o->kT, c->d_scal);
      dmpt_response(s, n, k, c->Mt32, c->eig, c->fill, o->kT, c->d_scal);
      grc |= pgemm('N', 'N', n, k, n, 1.f, c->C32, c->Mt32, 0.f, c->Zp32, 0);
      grc |= pgemm('N', 'T', n, n, k, 1.f, c->Zp32, c->C32, 0.f, c->A32, kCLower);
      grc |= pgemm('N', 'T', n, n, k, 1.f, c->C32, c->Zp32, 1.f, c->A32, kCLower);
      if (grc != 0) return set_error(c, DFTBGPU_ERR_CUDA, "tensor-core GEMM launch failed");
      add_lower_f_sym_d(s, n, c->rho_ref, c->A32, c->rho);
    } else if (form == kFormLow) {
      c->mixed_iters++;
      mark(c, kPhTransform);
      reduced_shift_f(s, g, c->L32, c->d_V, c->T32);
      gemm<float>(s, 'N', 'N', n, n, n, 1.f, c->Li32, n, c->T32, n, 0.f, c->C32, n, kALower | kBLower | kCLower);
      add_half_lower_f(s, n, c->A0_32, c->C32, c->A32);
      mark(c, kPhSytrd);
      const bool two_stage = use_twostage(n);
      if (two_stage)
        twostage_reduce<float>(s, n, c->A32, n, c->d32, c->e32, c->V32, n, c->wk32_ts, c->d_status);
      else
        sytrd_lower<float>(s, n, c->A32, n, c->d32, c->e32, c->tau32, c->V32, n, c->wk32_sytrd, c->d_status);
      mark(c, kPhStedc);
      if (stedc<float>(s, n, c->d32, c->e32, c->Z32, n, c->wk32_stedc, c->iwk_stedc, c->d_status) != 0)
        return set_error(c, DFTBGPU_ERR_ARGS, "stedc workspace layout error");
      convert_f2d(s, n, c->d32, c->eig);
      mark(c, kPhFermi);
      DG_CHECK(c, pick(&k));
      mark(c, kPhBack);
      if (k > 0) {
        if (two_stage)
          twostage_back<float>(s, n, k, c->Z32, n, c->V32, n, c->wk32_ts, c->d_status);
        else
          ormtr_left<float>(s, n, k, c->V32, n, c->tau32, c->Z32, n, c->wk32_ormtr);
        gemm<float>(s, 'T', 'N', n, k, n, 1.f, c->Li32, n, c->Z32, n, 0.f, c->C32, n, kAUpper);
      }
      mark(c, kPhDensity);
      if (k > 0) {
        scale_columns<float>(s, n, k, c->C32, n, c->fill, c->T32, n);
        gemm<float>(s, 'N', 'T', n, n, k, 1.f, c->T32, n, c->C32, n, 0.f, c->A32, n, kCLower);
        lower_f_to_sym_d(s, n, c->A32, c->rho);
      } else {
        set_zero(s, c->rho, (size_t)n * n);
      }
    } else {
      // reduced problem A = L^-1 H L^-T = A0 + 1/2 (B + B^T), B = L^-1 (diag(V) L)
      mark(c, kPhTransform);
      prof_flops(c, kPhTransform, (double)n * n * n);
      reduced_shift(s, g, c->Lc, c->d_V, c->T);
      dgemm(s, 'N', 'N', n, n, n, 1.0, c->Linv, n, c->T, n, 0.0, c->C, n, kALower | kBLower | kCLower);
      add_half_lower(s, n, c->A0, c->C, c->H);
      const bool reference = mixed && !verify;
      // FP64 back-transformation of the occupied vectors only; the reference's virtual vectors are
      // consumed in FP32 by the perturbative updates and are back-transformed in FP32 below
      DG_CHECK(c, eigensolve(c, n, c->H, pick, /*reduced=*/true, /*all_vectors=*/false));
      k = (int)h_scal[kSNLevels];
      mark(c, kPhDensity);
      prof_flops(c, kPhDensity, (double)n * n * k);
      DG_CHECK(c, density(c, n, k, c->fill, c->rho));
      if (reference) {
        // reference of the perturbative iterations: C (FP32), X = S C = L Y (FP32), rho, V.
        // Z holds Y for the first k columns and tridiagonal eigenvectors for the rest.
        mark(c, kPhPert);
        const size_t nk = (size_t)n * k;
        convert_d2f(s, (size_t)n * n, c->Z, c->Z32);
        convert_d2f(s, nk, c->C, c->C32);
        if (k < n) {
          convert_d2f(s, (size_t)n * n, c->Vh, c->T32);
          convert_d2f(s, (size_t)n, c->tau, c->tau32);
          ormtr_left<float>(s, n, n - k, c->T32, n, c->tau32, c->Z32 + nk, n, c->wk32_ormtr);
          gemm<float>(s, 'T', 'N', n, n - k, n, 1.f, c->Li32, n, c->Z32 + nk, n, 0.f, c->C32 + nk, n, kAUpper);
        }
        gemm<float>(s, 'N', 'N', n, n, n, 1.f, c->L32, n, c->Z32, n, 0.f, c->V32, n, kALower);
        DG_CUDA(c, cudaMemcpyAsync(c->rho_ref, c->rho, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, s));
        DG_CUDA(c, cudaMemcpyAsync(c->Vref, c->d_V, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
        k_ref = k;
      }
    }
    c->nlevels = k;
    mark(c, kPhMulliken);
    mulliken(s, g, c->rho, c->S, c->H0, c->qorb, c->d_qout, c->eorb, c->d_scal);
    potential(s, m, g, c->d_qout, c->d_q0, c->d_Vout);
    scc_energy(s, N, c->d_Vout, c->d_qout, c->d_q0, c->d_scal);
    mark(c, kPhBroyden);
    broyden_step(s, N, it, mix_calls + 1, o->min_iter, o->max_iter, o->scc_tol, o->mix_alpha, o->mix_omega0,
                 o->mix_min_weight, o->mix_max_weight, o->mix_weight_fac, c->bro, c->d_qin, c->d_qout, c->d_scal);
    mark(c, -1);
    DG_CUDA(c, cudaMemcpyAsync(h_scal, c->d_scal, sizeof(h_scal), cudaMemcpyDeviceToHost, s));
    DG_CUDA(c, cudaStreamSynchronize(s));
    DG_CUDA(c, cudaGetLastError());
    if (mixed && (tc_dgemm_error() || tc_gemm_error() || tc_fgemm_error()))
      return set_error(c, DFTBGPU_ERR_ITER_CAP, "tensor-core GEMM: a bounded wait timed out");
    g_tc_dgemm = false;
    g_tc_fgemm = false;
    flush_marks(c);
    c->hist_e.push_back(h_scal[kSEnonScc] + h_scal[kSEscc]);
    c->hist_err.push_back(h_scal[kSErr]);
    c->hist_prec.push_back(it_form == kFormFull ? (int)DFTBGPU_PREC_FP64
                                                : (it_form == kFormLow ? (int)DFTBGPU_PREC_MIXED
                                                                       : (int)DFTBGPU_ITER_PERTURB));
    c->hist_ms.push_back(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_it).count());
    conv = h_scal[kSConv] != 0.0;
    if (!conv && it != o->max_iter) ++mix_calls;
    if (mixed) {
      if (form == kFormLow) {
        // close enough in reduced precision (a converged FP32 state is re-evaluated, not accepted)
        if (conv || h_scal[kSErr] < switch_tol) form = kFormFull;
        conv = false;
      } else if (form == kFormFull) {
        if (!conv) {
          if (verify) {
            verify = false;   // the check failed: the next FULL iteration becomes a new reference
          } else {
            form = kFormPert;
            pert_run = 0;
          }
        }
      } else {
        // a converged perturbative state is re-evaluated by a FULL iteration at the same charges
        // (the mixer leaves q_in unchanged on convergence) that only needs the occupied vectors; a
        // long perturbative run renews the reference instead
        if (conv) {
          form = kFormFull;
          verify = true;
        } else if (++pert_run >= kMaxPertRun) {
          form = kFormFull;
        }
        conv = false;
      }
    }
    if (conv) break;
  }
  if (it > o->max_iter) it = o->max_iter;
  c->have_scc = true;
  c->have_w = false;
  if (energies) {
    energies->EnonSCC = h_scal[kSEnonScc];
    energies->Escc = h_scal[kSEscc];
    energies->Erep = h_scal[kSErep];
    energies->Eband = h_scal[kSEband];
    energies->TS = h_scal[kSTS];
    energies->E0 = h_scal[kSE0];
    energies->Etotal = h_scal[kSEnonScc] + h_scal[kSEscc] + h_scal[kSErep];
    energies->EMermin = energies->Etotal - h_scal[kSTS];
  }
  if (ef) *ef = h_scal[kSEf];
  if (eigen) DG_CUDA(c, cudaMemcpy(eigen, c->eig, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (filling) DG_CUDA(c, cudaMemcpy(filling, c->fill, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (q_out) DG_CUDA(c, cudaMemcpy(q_out, c->d_qout, sizeof(double) * N, cudaMemcpyDeviceToHost));
  if (n_iter) *n_iter = it;
  if (converged) *converged = conv ? 1 : 0;
  if (!conv && o->convergent_only)
    return set_error(c, DFTBGPU_ERR_SCC_NOT_CONVERGED, "SCC is NOT converged, maximal SCC iterations exceeded");
  return DFTBGPU_OK;
}

int dftbgpu_scc_history(const dftbgpu_ctx *c, int cap, double *energy, double *error, int *precision,
                        double *ms) {
  if (!c || cap < 0) return -1;
  const int n = (int)c->hist_err.size();
  for (int i = 0; i < n && i < cap; ++i) {
    if (energy) energy[i] = c->hist_e[i];
    if (error) error[i] = c->hist_err[i];
    if (precision) precision[i] = c->hist_prec[i];
    if (ms) ms[i] = c->hist_ms[i];
  }
  return n;
}

static int gradients_impl(dftbgpu_ctx *c, double *grad, bool dev) {
  if (!c || !grad) return DFTBGPU_ERR_ARGS;
  if (!c->have_scc) return set_error(c, DFTBGPU_ERR_STATE, "gradients: call dftbgpu_scc first");
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int n = c->norb;
  mark(c, kPhForces);
  prof_flops(c, kPhForces, (double)n * n * c->nlevels);
  energy_weights(s, c->nlevels, c->fill, c->eig, c->fe);
  g_tc_dgemm = c->scc_mixed && g_tc_dgemm_mixed;   // the mixed form's EDM product on the tensor cores
  const int rc_w = density(c, n, c->nlevels, c->fe, c->W);
  g_tc_dgemm = false;
  DG_CHECK(c, rc_w);
  c->have_w = true;
  GeomDev g = geom_view(c);
  ModelDev m = model_view(c);
  gradient_bands(s, m, g, c->rho, c->W, c->d_Vout, c->d_grad);
  gradient_dc_rep(s, m, g, c->d_qout, c->d_q0, c->d_grad);
  mark(c, -1);
  DG_CUDA(c, cudaGetLastError());
  if (dev) {
    DG_CUDA(c, cudaMemcpyAsync(grad, c->d_grad, sizeof(double) * 3 * c->natom, cudaMemcpyDeviceToDevice, s));
    DG_CUDA(c, cudaStreamSynchronize(s));
  } else {
    DG_CUDA(c, cudaMemcpyAsync(grad, c->d_grad, sizeof(double) * 3 * c->natom, cudaMemcpyDeviceToHost, s));
    DG_CUDA(c, cudaStreamSynchronize(s));
  }
  if (c->scc_mixed && tc_dgemm_error())   // read after the stream synchronised
    return set_error(c, DFTBGPU_ERR_ITER_CAP, "tensor-core GEMM: a bounded wait timed out");
  flush_marks(c);
  return DFTBGPU_OK;
}

int dftbgpu_grad_params(dftbgpu_ctx *c, double *dE_dskham, double *dE_dskover, double *dE_dhubbu) {
  if (!c) return DFTBGPU_ERR_ARGS;
  if (!c->have_scc) return set_error(c, DFTBGPU_ERR_STATE, "grad_params: call dftbgpu_scc first");
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int n = c->norb;
  if (!c->have_w) {
    energy_weights(s, c->nlevels, c->fill, c->eig, c->fe);
    DG_CHECK(c, density(c, n, c->nlevels, c->fe, c->W));
    c->have_w = true;
  }
  const size_t nt = (size_t)c->ham_len;
  double *d = nullptr;
  DG_CUDA(c, cudaMallocAsync((void **)&d, sizeof(double) * (2 * nt + c->nsp), s));
  DG_CUDA(c, cudaMemsetAsync(d, 0, sizeof(double) * (2 * nt + c->nsp), s));
  GeomDev g = geom_view(c);
  ModelDev m = model_view(c);
  sk_adjoint(s, m, g, c->d_pi, c->d_pj, c->npairs, c->rho, c->W, c->d_Vout, d, d + nt);
  hubbard_adjoint(s, m, g, c->d_qout, c->d_q0, d + 2 * nt);
  DG_CUDA(c, cudaGetLastError());
  if (dE_dskham) DG_CUDA(c, cudaMemcpyAsync(dE_dskham, d, sizeof(double) * nt, cudaMemcpyDeviceToHost, s));
  if (dE_dskover) DG_CUDA(c, cudaMemcpyAsync(dE_dskover, d + nt, sizeof(double) * nt, cudaMemcpyDeviceToHost, s));
  if (dE_dhubbu) DG_CUDA(c, cudaMemcpyAsync(dE_dhubbu, d + 2 * nt, sizeof(double) * c->nsp, cudaMemcpyDeviceToHost, s));
  DG_CUDA(c, cudaFreeAsync(d, s));
  DG_CUDA(c, cudaStreamSynchronize(s));
  return DFTBGPU_OK;
}

int dftbgpu_set_tensor_cores(int enable) {
  const int prev = g_tc_gemm ? 1 : 0;
  g_tc_gemm = enable != 0;
  return prev;
}

int dftbgpu_set_two_stage(int mode) {
  if (mode < 0 || mode > 2) return -1;
  return g_twostage.exchange(mode);
}

int dftbgpu_set_digit_gemm_kernel(int mode) {
  if (mode < 0 || mode > 1) return -1;
  return g_dg_kernel.exchange(mode);
}

int dftbgpu_set_panel_mode(int mode) {
  if (mode < 0 || mode > 2) return -1;
  return g_panel_mode.exchange(mode);
}

int dftbgpu_set_dc_staging(int enable) { return g_dc_stage.exchange(enable ? 1 : 0); }

int dftbgpu_set_fp64_emulation(int enable) {
  const int prev = g_tc_dgemm_mixed ? 1 : 0;
  g_tc_dgemm_mixed = enable != 0;
  return prev;
}

int dftbgpu_test_dgemm_tc(dftbgpu_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *a,
                          int lda, const double *b, int ldb, double beta, double *cm, int ldc, int flags) {
  if (!c || !a || !b || !cm || m <= 0 || n <= 0 || k <= 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  const size_t na = (size_t)lda * ((ta == 'N') ? k : m), nb = (size_t)ldb * ((tb == 'N') ? n : k),
               nc = (size_t)ldc * n;
  double *dA = nullptr, *dB = nullptr, *dC = nullptr;
  DG_CUDA(c, cudaMalloc((void **)&dA, na * sizeof(double)));
  DG_CUDA(c, cudaMalloc((void **)&dB, nb * sizeof(double)));
  DG_CUDA(c, cudaMalloc((void **)&dC, nc * sizeof(double)));
  DG_CUDA(c, cudaMemcpy(dA, a, na * sizeof(double), cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dB, b, nb * sizeof(double), cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dC, cm, nc * sizeof(double), cudaMemcpyHostToDevice));
  const int rc = tc_dgemm(c->stream, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, flags);
  DG_CUDA(c, cudaStreamSynchronize(c->stream));
  DG_CUDA(c, cudaMemcpy(cm, dC, nc * sizeof(double), cudaMemcpyDeviceToHost));
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  if (rc != 0) return set_error(c, DFTBGPU_ERR_CUDA, "tc_dgemm: %s", cudaGetErrorString((cudaError_t)rc));
  if (tc_dgemm_error()) return set_error(c, DFTBGPU_ERR_ITER_CAP, "tc_dgemm: a bounded wait timed out");
  return DFTBGPU_OK;
}

int dftbgpu_test_gemm_tc(dftbgpu_ctx *c, char ta, char tb, int m, int n, int k, float alpha, const float *a,
                         int lda, const float *b, int ldb, float beta, float *cm, int ldc, int flags) {
  if (!c || !a || !b || !cm || m <= 0 || n <= 0 || k <= 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  const size_t na = (size_t)lda * ((ta == 'N') ? k : m), nb = (size_t)ldb * ((tb == 'N') ? n : k),
               nc = (size_t)ldc * n;
  float *dA = nullptr, *dB = nullptr, *dC = nullptr;
  DG_CUDA(c, cudaMalloc((void **)&dA, na * sizeof(float)));
  DG_CUDA(c, cudaMalloc((void **)&dB, nb * sizeof(float)));
  DG_CUDA(c, cudaMalloc((void **)&dC, nc * sizeof(float)));
  DG_CUDA(c, cudaMemcpy(dA, a, na * sizeof(float), cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dB, b, nb * sizeof(float), cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dC, cm, nc * sizeof(float), cudaMemcpyHostToDevice));
  const int rc = tc_gemm(c->stream, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, flags);
  DG_CUDA(c, cudaStreamSynchronize(c->stream));
  DG_CUDA(c, cudaMemcpy(cm, dC, nc * sizeof(float), cudaMemcpyDeviceToHost));
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  if (rc != 0) return set_error(c, DFTBGPU_ERR_CUDA, "tc_gemm: %s", cudaGetErrorString((cudaError_t)rc));
  if (tc_gemm_error()) return set_error(c, DFTBGPU_ERR_ITER_CAP, "tc_gemm: a bounded wait timed out");
  return DFTBGPU_OK;
}

int dftbgpu_test_sgemm_digits(dftbgpu_ctx *c, char ta, char tb, int m, int n, int k, float alpha, const float *a,
                              int lda, const float *b, int ldb, float beta, float *cm, int ldc, int flags) {
  if (!c || !a || !b || !cm || m <= 0 || n <= 0 || k <= 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  const size_t na = (size_t)lda * ((ta == 'N') ? k : m), nb = (size_t)ldb * ((tb == 'N') ? n : k),
               nc = (size_t)ldc * n;
  float *dA = nullptr, *dB = nullptr, *dC = nullptr;
  DG_CUDA(c, cudaMalloc((void **)&dA, na * sizeof(float)));
  DG_CUDA(c, cudaMalloc((void **)&dB, nb * sizeof(float)));
  DG_CUDA(c, cudaMalloc((void **)&dC, nc * sizeof(float)));
  DG_CUDA(c, cudaMemcpy(dA, a, na * sizeof(float), cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dB, b, nb * sizeof(float), cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dC, cm, nc * sizeof(float), cudaMemcpyHostToDevice));
  const int rc = tc_fgemm(c->stream, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, flags);
  DG_CUDA(c, cudaStreamSynchronize(c->stream));
  DG_CUDA(c, cudaMemcpy(cm, dC, nc * sizeof(float), cudaMemcpyDeviceToHost));
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  if (rc != 0) return set_error(c, DFTBGPU_ERR_CUDA, "tc_fgemm: %s", cudaGetErrorString((cudaError_t)rc));
  if (tc_fgemm_error()) return set_error(c, DFTBGPU_ERR_ITER_CAP, "tc_fgemm: a bounded wait timed out");
  return DFTBGPU_OK;
}

int dftbgpu_set_fp32_emulation(int enable) {
  const int prev = g_tc_fgemm_mixed ? 1 : 0;
  g_tc_fgemm_mixed = enable != 0;
  return prev;
}

int dftbgpu_profile_enable(dftbgpu_ctx *c, int enable) {
  if (!c) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  flush_marks(c);
  for (auto &mk : c->marks) cudaEventDestroy(mk.second);
  c->marks.clear();
  if (enable) {
    for (int i = 0; i < kNPhase; ++i) {
      c->prof_ms[i] = 0.0;
      c->prof_flops[i] = 0.0;
      c->prof_calls[i] = 0;
    }
  }
  c->prof = enable != 0;
  g_gemm_prof.on = enable != 0;
  return DFTBGPU_OK;
}

int dftbgpu_profile_read(dftbgpu_ctx *c, int nphase, double *ms, double *flops, long long *calls) {
  if (!c || nphase < 0) return DFTBGPU_ERR_ARGS;
  int k = std::min(nphase, (int)kNPhase);
  for (int i = 0; i < k; ++i) {
    if (ms) ms[i] = c->prof_ms[i];
    if (flops) flops[i] = c->prof_flops[i];
    if (calls) calls[i] = c->prof_calls[i];
  }
  return k;
}

int dftbgpu_gradients(dftbgpu_ctx *c, double *grad) { return gradients_impl(c, grad, false); }
int dftbgpu_gradients_dev(dftbgpu_ctx *c, double *grad_dev) { return gradients_impl(c, grad_dev, true); }

int dftbgpu_n_orbitals(const dftbgpu_ctx *c, int *n_orb) {
  if (!c || !n_orb) return DFTBGPU_ERR_ARGS;
  *n_orb = c->norb;
  return DFTBGPU_OK;
}

int dftbgpu_get_orbital_populations(dftbgpu_ctx *c, double *q_orb) {
  if (!c || !q_orb) return DFTBGPU_ERR_ARGS;
  if (!c->have_scc) return set_error(c, DFTBGPU_ERR_STATE, "no SCC result");
  DG_CUDA(c, cudaMemcpy(q_orb, c->qorb, sizeof(double) * c->norb, cudaMemcpyDeviceToHost));
  return DFTBGPU_OK;
}

int dftbgpu_get_matrix(dftbgpu_ctx *c, int which, double *out) {
  if (!c || !out) return DFTBGPU_ERR_ARGS;
  if (!c->have_geom) return set_error(c, DFTBGPU_ERR_STATE, "no geometry");
  const double *src = nullptr;
  switch (which) {
    case 0: src = c->H0; break;
    case 1: src = c->S; break;
    case 2: src = c->have_scc ? c->rho : nullptr; break;
    case 3: src = nullptr; break;
    case 4: src = c->have_w ? c->W : nullptr; break;
    default: break;
  }
  if (!src) return set_error(c, DFTBGPU_ERR_STATE, "matrix %d not available", which);
  cudaSetDevice(c->device);
  DG_CUDA(c, cudaStreamSynchronize(c->stream));
  DG_CUDA(c, cudaMemcpy(out, src, sizeof(double) * (size_t)c->norb * c->norb, cudaMemcpyDeviceToHost));
  return DFTBGPU_OK;
}

int dftbgpu_sygvd(dftbgpu_ctx *c, int n, double *a, double *b, double *w) {
  if (!c || !a || !b || !w || n <= 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  DG_CHECK(c, ensure_orbitals(c, n));
  size_t nn = (size_t)n * n;
  DG_CUDA(c, cudaMemcpyAsync(c->H, a, sizeof(double) * nn, cudaMemcpyHostToDevice, s));
  DG_CUDA(c, cudaMemcpyAsync(c->Z, b, sizeof(double) * nn, cudaMemcpyHostToDevice, s));
  DG_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
  potrf_lower(s, n, c->Z, n, c->d_status);
  DG_CHECK(c, check_status(c, "sygvd Cholesky"));
  // the caller's b receives L; keep a copy because Z is reused by the tridiagonal solver
  DG_CUDA(c, cudaMemcpyAsync(b, c->Z, sizeof(double) * nn, cudaMemcpyDeviceToHost, s));
  trtri_lower(s, n, c->Z, n, c->Linv, n, c->T, (size_t)n * n);
  // the SCC state (if any) no longer matches the stored L^-1
  c->have_geom = false;
  c->have_scc = false;
  auto pick = [&](int *k) -> int {
    *k = n;
    return DFTBGPU_OK;
  };
  DG_CHECK(c, eigensolve(c, n, c->H, pick));
  DG_CHECK(c, check_status(c, "sygvd eigensolver"));
  DG_CUDA(c, cudaMemcpyAsync(w, c->eig, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  DG_CUDA(c, cudaMemcpyAsync(a, c->C, sizeof(double) * nn, cudaMemcpyDeviceToHost, s));
  DG_CUDA(c, cudaStreamSynchronize(s));
  return DFTBGPU_OK;
}

}  // extern "C"

extern "C" {

int dftbgpu_test_sgemm(dftbgpu_ctx *c, char ta, char tb, int m, int n, int k, float alpha, const float *a, int lda,
                       const float *b, int ldb, float beta, float *cm, int ldc, int flags) {
  if (!c || !a || !b || !cm || m <= 0 || n <= 0 || k <= 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  const size_t na = (size_t)lda * ((ta == 'N') ? k : m), nb = (size_t)ldb * ((tb == 'N') ? n : k),
               nc = (size_t)ldc * n;
  float *dA = nullptr, *dB = nullptr, *dC = nullptr;
  DG_CUDA(c, cudaMalloc((void **)&dA, na * sizeof(float)));
  DG_CUDA(c, cudaMalloc((void **)&dB, nb * sizeof(float)));
  DG_CUDA(c, cudaMalloc((void **)&dC, nc * sizeof(float)));
  DG_CUDA(c, cudaMemcpy(dA, a, na * sizeof(float), cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dB, b, nb * sizeof(float), cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dC, cm, nc * sizeof(float), cudaMemcpyHostToDevice));
  dg::gemm<float>(c->stream, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc, flags);
  DG_CUDA(c, cudaStreamSynchronize(c->stream));
  DG_CUDA(c, cudaGetLastError());
  DG_CUDA(c, cudaMemcpy(cm, dC, nc * sizeof(float), cudaMemcpyDeviceToHost));
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  return DFTBGPU_OK;
}

int dftbgpu_test_dgemm(dftbgpu_ctx *c, char ta, char tb, int m, int n, int k, double alpha, const double *a,
                       const double *b, double beta, double *cm, int flags) {
  if (!c || !a || !b || !cm || m <= 0 || n <= 0 || k < 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  bool TA = (ta == 'T' || ta == 't'), TB = (tb == 'T' || tb == 't');
  int lda = TA ? std::max(k, 1) : m, ldb = TB ? n : std::max(k, 1);
  size_t na = (size_t)lda * (TA ? m : std::max(k, 1)), nb = (size_t)ldb * (TB ? std::max(k, 1) : n);
  double *dA, *dB, *dC;
  DG_CUDA(c, cudaMalloc(&dA, na * 8));
  DG_CUDA(c, cudaMalloc(&dB, nb * 8));
  DG_CUDA(c, cudaMalloc(&dC, (size_t)m * n * 8));
  DG_CUDA(c, cudaMemcpy(dA, a, na * 8, cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dB, b, nb * 8, cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemcpy(dC, cm, (size_t)m * n * 8, cudaMemcpyHostToDevice));
  dg::dgemm(s, ta, tb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, m, flags);
  DG_CUDA(c, cudaStreamSynchronize(s));
  DG_CUDA(c, cudaMemcpy(cm, dC, (size_t)m * n * 8, cudaMemcpyDeviceToHost));
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  return DFTBGPU_OK;
}

int dftbgpu_test_tridiag(dftbgpu_ctx *c, int n, const double *a, double *d, double *e) {
  if (!c || !a || !d || !e || n <= 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  DG_CHECK(c, ensure_orbitals(c, n));
  DG_CUDA(c, cudaMemcpy(c->H, a, sizeof(double) * n * n, cudaMemcpyHostToDevice));
  sytrd_lower(s, n, c->H, n, c->dd, c->ee, c->tau, c->Vh, n, c->wk_sytrd, c->d_status);
  DG_CUDA(c, cudaGetLastError());
  DG_CUDA(c, cudaStreamSynchronize(s));
  DG_CUDA(c, cudaMemcpy(d, c->dd, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (n > 1) DG_CUDA(c, cudaMemcpy(e, c->ee, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost));
  c->have_geom = false;
  c->have_scc = false;
  return DFTBGPU_OK;
}

int dftbgpu_test_twostage(dftbgpu_ctx *c, int n, const double *a, int fp32, double *d, double *e, double *q) {
  if (!c || !a || !d || !e || !q || n <= 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const size_t nn = (size_t)n * n;
  DG_CHECK(c, ensure_orbitals(c, n));
  DG_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
  DG_CUDA(c, cudaMemcpyAsync(c->H, a, sizeof(double) * nn, cudaMemcpyHostToDevice, s));
  if (fp32) {
    DG_CHECK(c, ensure_mixed_buffers(c, n));
    convert_d2f(s, nn, c->H, c->A32);
    twostage_reduce<float>(s, n, c->A32, n, c->d32, c->e32, c->V32, n, c->wk32_ts, c->d_status);
    // Q = Q1 Q2 applied to the identity
    set_zero_t<float>(s, c->Z32, nn);
    identity_f(s, n, c->Z32);
    twostage_back<float>(s, n, n, c->Z32, n, c->V32, n, c->wk32_ts, c->d_status);
    convert_f2d(s, n, c->d32, c->dd);
    if (n > 1) convert_f2d(s, n - 1, c->e32, c->ee);
    convert_f2d(s, nn, c->Z32, c->Z);
  } else {
    const size_t need = twostage_work_size<double>(n);
    if (need > c->cap_ts64) {
      DG_CHECK(c, dev_alloc(c, &c->wk_ts, need));
      c->cap_ts64 = need;
    }
    twostage_reduce<double>(s, n, c->H, n, c->dd, c->ee, c->Vh, n, c->wk_ts, c->d_status);
    set_zero(s, c->Z, nn);
    identity_d(s, n, c->Z);
    twostage_back<double>(s, n, n, c->Z, n, c->Vh, n, c->wk_ts, c->d_status);
  }
  DG_CUDA(c, cudaGetLastError());
  DG_CHECK(c, check_status(c, "two-stage reduction"));
  DG_CUDA(c, cudaMemcpy(d, c->dd, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (n > 1) DG_CUDA(c, cudaMemcpy(e, c->ee, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost));
  DG_CUDA(c, cudaMemcpy(q, c->Z, sizeof(double) * nn, cudaMemcpyDeviceToHost));
  c->have_geom = false;
  c->have_scc = false;
  c->mixed_ready = false;
  return DFTBGPU_OK;
}

int dftbgpu_test_onestage(dftbgpu_ctx *c, int n, const double *a, int fp32, double *d, double *e, double *q) {
  if (!c || !a || !d || !e || !q || n <= 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const size_t nn = (size_t)n * n;
  DG_CHECK(c, ensure_orbitals(c, n));
  DG_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
  DG_CUDA(c, cudaMemcpyAsync(c->H, a, sizeof(double) * nn, cudaMemcpyHostToDevice, s));
  if (fp32) {
    DG_CHECK(c, ensure_mixed_buffers(c, n));
    convert_d2f(s, nn, c->H, c->A32);
    sytrd_lower<float>(s, n, c->A32, n, c->d32, c->e32, c->tau32, c->V32, n, c->wk32_sytrd, c->d_status);
    set_zero_t<float>(s, c->Z32, nn);
    identity_f(s, n, c->Z32);
    ormtr_left<float>(s, n, n, c->V32, n, c->tau32, c->Z32, n, c->wk32_ormtr);
    convert_f2d(s, n, c->d32, c->dd);
    if (n > 1) convert_f2d(s, n - 1, c->e32, c->ee);
    convert_f2d(s, nn, c->Z32, c->Z);
  } else {
    sytrd_lower(s, n, c->H, n, c->dd, c->ee, c->tau, c->Vh, n, c->wk_sytrd, c->d_status);
    set_zero(s, c->Z, nn);
    identity_d(s, n, c->Z);
    ormtr_left(s, n, n, c->Vh, n, c->tau, c->Z, n, c->wk_ormtr);
  }
  DG_CUDA(c, cudaGetLastError());
  DG_CHECK(c, check_status(c, "one-stage reduction"));
  DG_CUDA(c, cudaMemcpy(d, c->dd, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (n > 1) DG_CUDA(c, cudaMemcpy(e, c->ee, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost));
  DG_CUDA(c, cudaMemcpy(q, c->Z, sizeof(double) * nn, cudaMemcpyDeviceToHost));
  c->have_geom = false;
  c->have_scc = false;
  c->mixed_ready = false;
  return DFTBGPU_OK;
}

int dftbgpu_test_stedc(dftbgpu_ctx *c, int n, double *d, const double *e, double *q) {
  if (!c || !d || !q || n <= 0) return DFTBGPU_ERR_ARGS;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  DG_CHECK(c, ensure_orbitals(c, n));
  DG_CUDA(c, cudaMemcpy(c->dd, d, sizeof(double) * n, cudaMemcpyHostToDevice));
  if (n > 1) DG_CUDA(c, cudaMemcpy(c->ee, e, sizeof(double) * (n - 1), cudaMemcpyHostToDevice));
  DG_CUDA(c, cudaMemset(c->d_status, 0, sizeof(int)));
  if (stedc(s, n, c->dd, c->ee, c->Z, n, c->wk_stedc, c->iwk_stedc, c->d_status) != 0)
    return set_error(c, DFTBGPU_ERR_ARGS, "stedc layout");
  DG_CHECK(c, check_status(c, "stedc"));
  DG_CUDA(c, cudaMemcpy(d, c->dd, sizeof(double) * n, cudaMemcpyDeviceToHost));
  DG_CUDA(c, cudaMemcpy(q, c->Z, sizeof(double) * n * n, cudaMemcpyDeviceToHost));
  c->have_geom = false;
  c->have_scc = false;
  return DFTBGPU_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------ batched form
extern "C" {

int dftbgpu_batch_set_geometries(dftbgpu_ctx *c, int nmol, const int *atom_off, const double *coords,
                                 const int *species) {
  if (!c) return DFTBGPU_ERR_ARGS;
  if (!c->have_model) return set_error(c, DFTBGPU_ERR_STATE, "batch: no model set");
  cudaSetDevice(c->device);
  if (!c->batch) c->batch = new BatchState();
  char msg[256] = {0};
  const int rc = batch_set_geometries(c->stream, *c->batch, model_view(c), c->h_sp, c->sk_cut_max, nmol, atom_off,
                                      coords, species, false, msg, sizeof(msg));
  if (rc != DFTBGPU_OK) return set_error(c, rc, "%s", msg);
  return DFTBGPU_OK;
}

int dftbgpu_batch_set_geometries_dev(dftbgpu_ctx *c, int nmol, const int *atom_off, const double *coords_dev,
                                     const int *species) {
  if (!c) return DFTBGPU_ERR_ARGS;
  if (!c->have_model) return set_error(c, DFTBGPU_ERR_STATE, "batch: no model set");
  cudaSetDevice(c->device);
  if (!c->batch) c->batch = new BatchState();
  char msg[256] = {0};
  const int rc = batch_set_geometries(c->stream, *c->batch, model_view(c), c->h_sp, c->sk_cut_max, nmol, atom_off,
                                      coords_dev, species, true, msg, sizeof(msg));
  if (rc != DFTBGPU_OK) return set_error(c, rc, "%s", msg);
  return DFTBGPU_OK;
}

int dftbgpu_batch_scc(dftbgpu_ctx *c, const dftbgpu_scc_opts *o, dftbgpu_energies *energies, double *q_out,
                      int *n_iter, int *converged) {
  if (!c || !o) return DFTBGPU_ERR_ARGS;
  if (!c->batch || !c->batch->have_geom) return set_error(c, DFTBGPU_ERR_STATE, "batch: no geometries set");
  if (o->max_iter < 1 || o->max_iter > 150) return set_error(c, DFTBGPU_ERR_ARGS, "scc: max_iter must be in 1..150");
  if (!(o->kT > 0.0)) return set_error(c, DFTBGPU_ERR_ARGS, "scc: kT must be > 0 (Fermi filling)");
  if (o->precision != DFTBGPU_PREC_FP64 && o->precision != DFTBGPU_PREC_MIXED)
    return set_error(c, DFTBGPU_ERR_ARGS, "scc: unknown precision form %d", o->precision);
  cudaSetDevice(c->device);
  BatchState &b = *c->batch;
  BatchOpts bo{o->kT, o->scc_tol, o->mix_alpha, o->mix_omega0, o->mix_min_weight, o->mix_max_weight,
               o->mix_weight_fac, o->net_charge, (o->mixed_switch_tol > 0.0) ? o->mixed_switch_tol : 1e-3,
               o->max_iter, o->min_iter, o->precision == DFTBGPU_PREC_MIXED ? 1 : 0};
  char msg[256] = {0};
  int rc = batch_scc(c->stream, b, model_view(c), bo, msg, sizeof(msg));
  if (rc != DFTBGPU_OK) return set_error(c, rc, "%s", msg);
  std::vector<MolState> st(b.nmol);
  DG_CUDA(c, cudaMemcpy(st.data(), b.d.st, sizeof(MolState) * b.nmol, cudaMemcpyDeviceToHost));
  if (q_out) DG_CUDA(c, cudaMemcpy(q_out, b.d.qout, sizeof(double) * b.natom, cudaMemcpyDeviceToHost));
  int first_bad = -1, bad_status = 0, first_unconv = -1;
  for (int i = 0; i < b.nmol; ++i) {
    const MolState &m = st[i];
    if (energies) {
      dftbgpu_energies &e = energies[i];
      e.EnonSCC = m.enonscc;
      e.Escc = m.escc;
      e.Erep = m.erep;
      e.Eband = m.eband;
      e.TS = m.ts;
      e.E0 = m.e0;
      e.Etotal = m.enonscc + m.escc + m.erep;
      e.EMermin = e.Etotal - m.ts;
    }
    if (n_iter) n_iter[i] = m.n_iter;
    if (converged) converged[i] = m.conv;
    if (m.status != 0 && first_bad < 0) {
      first_bad = i;
      bad_status = m.status;
    }
    if (!m.conv && first_unconv < 0) first_unconv = i;
  }
  if (first_bad >= 0) {
    if (bad_status == kDevIterCap)
      return set_error(c, DFTBGPU_ERR_ITER_CAP, "batch: molecule %d: eigensolver iteration cap reached", first_bad);
    if (bad_status == kDevFermiFail)
      return set_error(c, DFTBGPU_ERR_FERMI, "batch: molecule %d: Fermi level search did not converge", first_bad);
    return set_error(c, DFTBGPU_ERR_CUDA, "batch: molecule %d: device status %d", first_bad, bad_status);
  }
  if (first_unconv >= 0 && o->convergent_only)
    return set_error(c, DFTBGPU_ERR_SCC_NOT_CONVERGED, "batch: molecule %d: SCC is NOT converged", first_unconv);
  return DFTBGPU_OK;
}

int dftbgpu_batch_gradients(dftbgpu_ctx *c, double *grad) {
  if (!c || !grad) return DFTBGPU_ERR_ARGS;
  if (!c->batch) return set_error(c, DFTBGPU_ERR_STATE, "batch: no geometries set");
  cudaSetDevice(c->device);
  BatchState &b = *c->batch;
  char msg[256] = {0};
  const int rc = batch_gradients(c->stream, b, model_view(c), msg, sizeof(msg));
  if (rc != DFTBGPU_OK) return set_error(c, rc, "%s", msg);
  DG_CUDA(c, cudaMemcpyAsync(grad, b.d.grad, sizeof(double) * 3 * b.natom, cudaMemcpyDeviceToHost, c->stream));
  DG_CUDA(c, cudaStreamSynchronize(c->stream));
  return DFTBGPU_OK;
}

}  // extern "C"
