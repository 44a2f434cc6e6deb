// Shared definitions of the dftbgpu CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/dftbgpu.h"

namespace dg {

constexpr int kMaxShell = 4;
constexpr int kMaxOrb = 9;          // s, p, d per atom (f is not supported on this path)
constexpr int kMaxInt = 14;         // integrals per ordered pair for s, p, d shells (spd-spd)

struct SpeciesDev {
  int n_shell;
  int ang[kMaxShell];
  int n_orb;
  double onsite[kMaxShell];
  double hubbu;
  double occ[kMaxShell];
};

struct PairDev {
  double dist;            // grid spacing
  int rows;               // grid rows (row j <-> r = (j+1) dist)
  int n_int;              // integrals
  long long off_ham;      // offset into the table array (column-major rows x n_int)
  long long off_over;
  long long off_rep;      // offset into the repulsive data
  int n_spline;
  double rep_cut;
  double sk_cut;          // rows*dist + 1 Bohr tail
  double gamma_cut;       // short-gamma cutoff for this species pair
  // tail (5th-order polynomial) coefficients per integral for H and S: y1, y1', y1''
  double tail_h[3][kMaxInt];
  double tail_s[3][kMaxInt];
};

struct Ctx;

// Error helpers: return a status with a message stored in the context.
int set_error(Ctx *c, int code, const char *fmt, ...);

#define DG_CUDA(c, call)                                                                 \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return ::dg::set_error((c), DFTBGPU_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__,  \
                             #call, cudaGetErrorString(e_));                             \
  } while (0)

#define DG_CHECK(c, stat)                \
  do {                                   \
    int s_ = (stat);                     \
    if (s_ != DFTBGPU_OK) return s_;     \
  } while (0)

// Count of kernel launches issued by this library (for launch accounting).
extern std::atomic<long long> g_launches;
inline void count_launch(long long n = 1) { g_launches += n; }

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Raises the dynamic shared-memory limit of kernel fn to `bytes` on the current device. The limit is
// a per-device property of the function, so it is recorded per (device, kernel): a process with
// contexts on several GPUs sets it on each of them once.
inline cudaError_t ensure_dyn_smem(const void *fn, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, int> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(dev, fn);
  const auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done[key] = bytes;
  return e;
}

// Profiling phases (order documented in include/dftbgpu.h, dftbgpu_profile_enable).
enum Phase : int {
  kPhH0S = 0, kPhPot, kPhTransform, kPhSytrd, kPhStedc, kPhFermi, kPhBack, kPhDensity, kPhMulliken,
  kPhBroyden, kPhForces, kPhPert, kPhGemm, kPhGemm32, kPhGemmTc,
  // single kernels, timed launch by launch (work = algorithmic bytes or tasks, see the header)
  kPhKSytrdPanel, kPhKPanelQr, kPhKChase, kPhKBackQ2, kPhKSytrdPanel32,
  kNPhase
};

// Device-side status word codes (written by bounded device loops instead of spinning/trapping).
enum DevStatus : int {
  kDevOk = 0,
  kDevNotPosDef = 1,
  kDevIterCap = 2,
  kDevFermiFail = 3,
};

}  // namespace dg
