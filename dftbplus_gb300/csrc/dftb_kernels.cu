// DFTB hot-path kernels: GPU neighbour list, SK integrals and rotations, H0/S, electrostatic
// potentials, Hamiltonian assembly, Mulliken analysis, Fermi filling, Broyden mixing, energies and
// the FD-based force contraction. FP64 throughout (the plain drop-in form).
#include <cfloat>

#include "dftb_device.cuh"

namespace dg {

// ------------------------------------------------------------------------------ neighbour list
__global__ void pair_count_kernel(GeomDev g, double cut2, int *count) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (i >= g.natom) return;
  double xi = g.xyz[3 * i], yi = g.xyz[3 * i + 1], zi = g.xyz[3 * i + 2];
  int c = 0;
  for (int j = i + 1 + lane; j < g.natom; j += 32) {
    double dx = g.xyz[3 * j] - xi, dy = g.xyz[3 * j + 1] - yi, dz = g.xyz[3 * j + 2] - zi;
    if (dx * dx + dy * dy + dz * dz <= cut2) ++c;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0) count[i] = c;
}

// exclusive scan of count[0..n) into start[0..n], single CTA
__global__ void scan_kernel(int n, const int *count, int *start) {
  __shared__ int sh[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    int i = base + threadIdx.x;
    int v = (i < n) ? count[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      int t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) start[i] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += sh[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) start[n] = carry;
}

__global__ void pair_fill_kernel(GeomDev g, double cut2, const int *start, int *pi, int *pj) {
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (i >= g.natom) return;
  double xi = g.xyz[3 * i], yi = g.xyz[3 * i + 1], zi = g.xyz[3 * i + 2];
  int pos = start[i];
  for (int j0 = i + 1; j0 < g.natom; j0 += 32) {
    int j = j0 + lane;
    bool in = false;
    if (j < g.natom) {
      double dx = g.xyz[3 * j] - xi, dy = g.xyz[3 * j + 1] - yi, dz = g.xyz[3 * j + 2] - zi;
      in = dx * dx + dy * dy + dz * dz <= cut2;
    }
    unsigned b = __ballot_sync(0xffffffffu, in);
    if (in) {
      int k = pos + __popc(b & ((1u << lane) - 1u));
      pi[k] = i;
      pj[k] = j;
    }
    pos += __popc(b);
  }
}

void build_pairs(cudaStream_t s, const GeomDev &g, double cutoff, int *count, int *start, int *pi, int *pj,
                 size_t cap, int *npairs_host) {
  double cut2 = cutoff * cutoff;
  int blocks = ceil_div((long long)g.natom * 32, 256);
  pair_count_kernel<<<blocks, 256, 0, s>>>(g, cut2, count);
  scan_kernel<<<1, 1024, 0, s>>>(g.natom, count, start);
  count_launch(2);
  cudaMemcpyAsync(npairs_host, start + g.natom, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  // the caller grows the pair arrays and calls again when they are too small
  if (*npairs_host > 0 && (size_t)*npairs_host <= cap) {
    pair_fill_kernel<<<blocks, 256, 0, s>>>(g, cut2, start, pi, pj);
    count_launch();
  }
}

// ------------------------------------------------------------------------------ H0 / S
__global__ void onsite_kernel(ModelDev M, GeomDev g, double *H0, double *S) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= g.natom) return;
  const SpeciesDev &sp = M.sp[g.species[a]];
  int o = g.orb_off[a];
  int k = 0;
  for (int sh = 0; sh < sp.n_shell; ++sh)
    for (int q = 0; q < 2 * sp.ang[sh] + 1; ++q, ++k) {
      size_t idx = (size_t)(o + k) * (g.norb + 1);
      H0[idx] = sp.onsite[sh];
      S[idx] = 1.0;
    }
}

__global__ void __launch_bounds__(128) h0s_kernel(ModelDev M, GeomDev g, const int *pi, const int *pj,
                                                  int npairs, double *H0, double *S) {
  __shared__ WarpSk ws_all[4];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p = blockIdx.x * 4 + w;
  if (p >= npairs) return;
  WarpSk &ws = ws_all[w];
  const int i = pi[p], j = pj[p];
  const int si = g.species[i], sj = g.species[j];
  const double vx = g.xyz[3 * j] - g.xyz[3 * i];
  const double vy = g.xyz[3 * j + 1] - g.xyz[3 * i + 1];
  const double vz = g.xyz[3 * j + 2] - g.xyz[3 * i + 2];
  eval_blocks(M, si, sj, vx, vy, vz, ws, lane);
  const int oi = g.orb_off[i], oj = g.orb_off[j];
  const int ni = M.sp[si].n_orb, nj = M.sp[sj].n_orb;
  const size_t n = g.norb;
  for (int idx = lane; idx < ni * nj; idx += 32) {
    int b = idx % nj, a = idx / nj;
    double hv = ws.blk[0][b][a], sv = ws.blk[1][b][a];
    H0[(oj + b) + (oi + a) * n] = hv;
    H0[(oi + a) + (oj + b) * n] = hv;
    S[(oj + b) + (oi + a) * n] = sv;
    S[(oi + a) + (oj + b) * n] = sv;
  }
}

void build_h0_s(cudaStream_t s, const ModelDev &m, const GeomDev &g, const int *pi, const int *pj,
                int npairs, double *H0, double *S) {
  size_t nn = (size_t)g.norb * g.norb;
  cudaMemsetAsync(H0, 0, nn * sizeof(double), s);
  cudaMemsetAsync(S, 0, nn * sizeof(double), s);
  onsite_kernel<<<ceil_div(g.natom, 128), 128, 0, s>>>(m, g, H0, S);
  count_launch();
  if (npairs > 0) {
    h0s_kernel<<<ceil_div(npairs, 4), 128, 0, s>>>(m, g, pi, pj, npairs, H0, S);
    count_launch();
  }
}

// V_A = sum_{B != A} dq_B / r_AB - sum_{B: r <= rc} gamma_short(r_AB) dq_B (coulomb.F90:537-585,
// shortgamma.F90:860-936; on-site gamma_short(0) = -U).
__global__ void potential_kernel(ModelDev M, GeomDev g, const double *q, const double *q0, double *V) {
  int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (a >= g.natom) return;
  const double xa = g.xyz[3 * a], ya = g.xyz[3 * a + 1], za = g.xyz[3 * a + 2];
  const int sa = g.species[a];
  const double ua = M.sp[sa].hubbu;
  double s = 0.0;
  for (int b = lane; b < g.natom; b += 32) {
    double dq = q[b] - q0[b];
    if (b == a) {
      s -= exp_gamma(0.0, ua, ua) * dq;
      continue;
    }
    double dx = xa - g.xyz[3 * b], dy = ya - g.xyz[3 * b + 1], dz = za - g.xyz[3 * b + 2];
    double r2 = dx * dx + dy * dy + dz * dz;
    double r = sqrt(r2);
    s += dq / r;
    const int sb = g.species[b];
    double rc = M.pair[sa * M.nsp + sb].gamma_cut;
    if (r2 <= rc * rc + kTolSameDist * kTolSameDist) s -= exp_gamma(r, M.sp[sb].hubbu, ua) * dq;
  }
  s = warp_sum(s);
  if (lane == 0) V[a] = s;
}

void potential(cudaStream_t s, const ModelDev &m, const GeomDev &g, const double *q, const double *q0,
               double *V) {
  potential_kernel<<<ceil_div((long long)g.natom * 32, 256), 256, 0, s>>>(m, g, q, q0, V);
  count_launch();
}

// ------------------------------------------------------------------------------ H assembly
__global__ void assemble_h_kernel(int n, const int *orb_atom, const double *H0, const double *S,
                                  const double *V, double *H) {
  int j = blockIdx.y;
  double vj = V[orb_atom[j]];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    size_t idx = i + (size_t)j * n;
    H[idx] = H0[idx] + 0.5 * S[idx] * (V[orb_atom[i]] + vj);
  }
}

__global__ void orb_atom_kernel(GeomDev g, int *orb_atom) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= g.natom) return;
  for (int o = g.orb_off[a]; o < g.orb_off[a + 1]; ++o) orb_atom[o] = a;
}

// DL = diag(V_orb) L on the lower triangle (zero above): the SCC shift enters the reduced problem
// only through B = L^-1 (D L), since L^-1 (H0 + 1/2 (D S + S D)) L^-T = A0 + 1/2 (B + B^T).
__global__ void scale_rows_lower_kernel(int n, const int *orb_atom, const double *L, const double *V,
                                        double *DL) {
  int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    size_t idx = i + (size_t)j * n;
    DL[idx] = (i >= j) ? V[orb_atom[i]] * L[idx] : 0.0;
  }
}

// A (lower) = A0 + 1/2 (B + B^T) for lower-triangular B: off-diagonal A0 + B/2, diagonal A0 + B.
__global__ void add_half_lower_kernel(int n, const double *A0, const double *B, double *A) {
  int j = blockIdx.y;
  for (int i = j + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    size_t idx = i + (size_t)j * n;
    A[idx] = A0[idx] + ((i == j) ? B[idx] : 0.5 * B[idx]);
  }
}

void reduced_shift(cudaStream_t s, const GeomDev &g, const double *L, const double *V, double *DL) {
  const int *orb_atom = g.orb_off + g.natom + 1;
  dim3 grid(std::min(ceil_div(g.norb, 256), 4), g.norb);
  scale_rows_lower_kernel<<<grid, 256, 0, s>>>(g.norb, orb_atom, L, V, DL);
  count_launch();
}

void add_half_lower(cudaStream_t s, int n, const double *A0, const double *B, double *A) {
  dim3 grid(std::min(ceil_div(n, 256), 4), n);
  add_half_lower_kernel<<<grid, 256, 0, s>>>(n, A0, B, A);
  count_launch();
}

// FP32 counterparts for the reduced-precision SCC iterations of the mixed form.
__global__ void scale_rows_lower_f_kernel(int n, const int *orb_atom, const float *L, const double *V, float *DL) {
  int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    size_t idx = i + (size_t)j * n;
    DL[idx] = (i >= j) ? (float)V[orb_atom[i]] * L[idx] : 0.0f;
  }
}
__global__ void add_half_lower_f_kernel(int n, const float *A0, const float *B, float *A) {
  int j = blockIdx.y;
  for (int i = j + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    size_t idx = i + (size_t)j * n;
    A[idx] = A0[idx] + ((i == j) ? B[idx] : 0.5f * B[idx]);
  }
}
__global__ void d2f_kernel(size_t n, const double *x, float *y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
__global__ void f2d_kernel(size_t n, const float *x, double *y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}
// full symmetric FP64 matrix from the lower triangle of an FP32 one
__global__ void lower_f_to_sym_d_kernel(int n, const float *A, double *B) {
  int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    B[i + (size_t)j * n] = (double)((i >= j) ? A[i + (size_t)j * n] : A[j + (size_t)i * n]);
}

void reduced_shift_f(cudaStream_t s, const GeomDev &g, const float *L, const double *V, float *DL) {
  const int *orb_atom = g.orb_off + g.natom + 1;
  dim3 grid(std::min(ceil_div(g.norb, 256), 4), g.norb);
  scale_rows_lower_f_kernel<<<grid, 256, 0, s>>>(g.norb, orb_atom, L, V, DL);
  count_launch();
}
void add_half_lower_f(cudaStream_t s, int n, const float *A0, const float *B, float *A) {
  dim3 grid(std::min(ceil_div(n, 256), 4), n);
  add_half_lower_f_kernel<<<grid, 256, 0, s>>>(n, A0, B, A);
  count_launch();
}
void convert_d2f(cudaStream_t s, size_t n, const double *x, float *y) {
  d2f_kernel<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(n, x, y);
  count_launch();
}
void convert_f2d(cudaStream_t s, size_t n, const float *x, double *y) {
  f2d_kernel<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(n, x, y);
  count_launch();
}
void lower_f_to_sym_d(cudaStream_t s, int n, const float *A, double *B) {
  dim3 grid(std::min(ceil_div(n, 256), 4), n);
  lower_f_to_sym_d_kernel<<<grid, 256, 0, s>>>(n, A, B);
  count_launch();
}

// ------------------------------------------------------------- density-matrix perturbation
// First-order change of the density matrix of H C = S C eps under H -> H + 1/2 (S D + D S),
// D = diag(dV): with X = S C (so C^T S C = I), M = C^T dH C = 1/2 (X^T D C + C^T D X) and
// dP_ij = K_ij (M_ij - dmu delta_ij), K_ij = (f_i - f_j) / (eps_i - eps_j) (f' on the diagonal and
// for degenerate pairs), drho = C dP C^T. Only rows/columns with f > 0 (i < k) contribute.
__global__ void dmpt_scale_kernel(int n, const int *orb_atom, const double *V, const double *Vref,
                                  const float *C, const float *X, float *DC, float *DX) {
  const int j = blockIdx.y;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n; l += gridDim.x * blockDim.x) {
    const int a = orb_atom[l];
    const float dv = (float)(V[a] - Vref[a]);
    const size_t o = l + (size_t)j * n;
    DC[o] = dv * C[o];
    DX[o] = dv * X[o];
  }
}

__device__ __forceinline__ double fermi_deriv(double f, double kT) {
  // f = 2 / (1 + exp((e - mu) / kT))  =>  df/de = -f (2 - f) / (2 kT)
  return -f * (2.0 - f) / (2.0 * kT);
}

__global__ void dmpt_dmu_kernel(int n, int k, const float *Mt, const double *fill, double kT, double *scal) {
  __shared__ double sn[256], sd[256];
  double num = 0.0, den = 0.0;
  for (int i = threadIdx.x; i < k; i += 256) {
    const double fp = fermi_deriv(fill[i], kT);
    num = fma(fp, (double)Mt[i + (size_t)i * n], num);
    den += fp;
  }
  sn[threadIdx.x] = num;
  sd[threadIdx.x] = den;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sn[threadIdx.x] += sn[threadIdx.x + o];
      sd[threadIdx.x] += sd[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) scal[kSDmu] = (fabs(sd[0]) > 1e-300) ? sn[0] / sd[0] : 0.0;
}

__global__ void dmpt_response_kernel(int n, int k, float *Mt, const double *eig, const double *fill, double kT,
                                     const double *scal) {
  const int i = blockIdx.y;
  const double fi = fill[i], ei = eig[i], dmu = scal[kSDmu];
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const size_t o = j + (size_t)i * n;
    double m = (double)Mt[o];
    double K;
    if (j == i) {
      K = fermi_deriv(fi, kT);
      m -= dmu;
    } else {
      const double de = ei - eig[j];
      if (fabs(de) > 1e-9) K = (fi - fill[j]) / de;
      else K = fermi_deriv(0.5 * (fi + fill[j]), kT);
    }
    double v = K * m;
    if (j < k) v *= 0.5;
    Mt[o] = (float)v;
  }
}

__global__ void add_lower_f_sym_d_kernel(int n, const double *Bref, const float *D, double *B) {
  const int j = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const size_t o = i + (size_t)j * n;
    B[o] = Bref[o] + (double)((i >= j) ? D[o] : D[j + (size_t)i * n]);
  }
}

void dmpt_scale(cudaStream_t s, const GeomDev &g, const double *V, const double *Vref, const float *C,
                const float *X, float *DC, float *DX) {
  const int *orb_atom = g.orb_off + g.natom + 1;
  dim3 grid(std::min(ceil_div(g.norb, 256), 4), g.norb);
  dmpt_scale_kernel<<<grid, 256, 0, s>>>(g.norb, orb_atom, V, Vref, C, X, DC, DX);
  count_launch();
}
void dmpt_dmu(cudaStream_t s, int n, int k, const float *Mt, const double *fill, double kT, double *scal) {
  dmpt_dmu_kernel<<<1, 256, 0, s>>>(n, k, Mt, fill, kT, scal);
  count_launch();
}
void dmpt_response(cudaStream_t s, int n, int k, float *Mt, const double *eig, const double *fill, double kT,
                   const double *scal) {
  if (k <= 0) return;
  dim3 grid(std::min(ceil_div(n, 256), 4), k);
  dmpt_response_kernel<<<grid, 256, 0, s>>>(n, k, Mt, eig, fill, kT, scal);
  count_launch();
}
void add_lower_f_sym_d(cudaStream_t s, int n, const double *Bref, const float *D, double *B) {
  dim3 grid(std::min(ceil_div(n, 256), 4), n);
  add_lower_f_sym_d_kernel<<<grid, 256, 0, s>>>(n, Bref, D, B);
  count_launch();
}

void assemble_h(cudaStream_t s, const GeomDev &g, const double *H0, const double *S, const double *V,
                double *H) {
  // orb_off holds natom+1 entries followed by norb orbital->atom entries (see api.cu)
  const int *orb_atom = g.orb_off + g.natom + 1;
  dim3 grid(std::min(ceil_div(g.norb, 256), 4), g.norb);
  assemble_h_kernel<<<grid, 256, 0, s>>>(g.norb, orb_atom, H0, S, V, H);
  count_launch();
}

// ------------------------------------------------------------------------------ reductions
// block-wide compensated sum (all threads get the result); blockDim.x == 1024
__device__ double block_csum(Comp v, double *sh_s, double *sh_c) {
  // fold the compensation, then reduce (s, c) pairs with neumaier across the tree
  for (int o = 16; o > 0; o >>= 1) {
    double os = __shfl_xor_sync(0xffffffffu, v.s, o);
    double oc = __shfl_xor_sync(0xffffffffu, v.c, o);
    neumaier(v, os);
    v.c += oc;
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sh_s[w] = v.s; sh_c[w] = v.c; }
  __syncthreads();
  if (w == 0) {
    Comp u = {sh_s[lane], sh_c[lane]};
    for (int o = 16; o > 0; o >>= 1) {
      double os = __shfl_xor_sync(0xffffffffu, u.s, o);
      double oc = __shfl_xor_sync(0xffffffffu, u.c, o);
      neumaier(u, os);
      u.c += oc;
    }
    if (lane == 0) sh_s[32] = u.s + u.c;
  }
  __syncthreads();
  double r = sh_s[32];
  __syncthreads();
  return r;
}

// ------------------------------------------------------------------------------ Fermi filling
__device__ double electron_count(int n, const double *eig, double ef, double beta, double *sh_s,
                                 double *sh_c) {
  Comp c = {0.0, 0.0};
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double x = (eig[j] - ef) * beta;
    neumaier(c, 1.0 / (1.0 + exp(x)));
  }
  return block_csum(c, sh_s, sh_c);
}

// etemp.F90:59-191 (Efilling, Fermi distribution, one spin channel with N_el/2, x2 afterwards as
// in main.F90:4544-4649). One CTA of 1024 threads; bounded loops.
__global__ void __launch_bounds__(1024) fermi_kernel(int n, const double *eig, double nel_total, double kT,
                                                     double *fill, double *scal) {
  __shared__ double sh_s[33], sh_c[33];
  __shared__ int sh_i;
  const double nel = 0.5 * nel_total;
  const double beta = 1.0 / kT;
  const double eps2 = 2.0 * kEps;
  double ef;
  int status = 0;
  bool rescale = false;
  double ne_final = nel;
  if ((double)n <= nel) {
    ef = eig[n - 1] + 1000.0 * (kT + (double)FLT_EPSILON);
  } else {
    bool done = false;
    if (fabs(nel - rint(nel)) <= kElecTol) {
      int nocc = (int)ceil(nel - 1e-12);
      if (nocc < 1) nocc = 1;
      int lumo = min(n, nocc + 1) - 1;
      ef = 0.5 * (eig[lumo] + eig[nocc - 1]);
      double ne = electron_count(n, eig, ef, beta, sh_s, sh_c);
      if (fabs(nel - ne) <= kElecTolMax) done = true;
    }
    if (!done) {
      double up = eig[n - 1] + 0.01, lo = eig[0] - 0.01;
      double nmax = electron_count(n, eig, up, beta, sh_s, sh_c);
      double nmin = electron_count(n, eig, lo, beta, sh_s, sh_c);
      int guard = 0;
      while (nmin > nel && guard++ < 200) {
        lo = 2.0 * (lo - up) + lo;
        nmin = electron_count(n, eig, lo, beta, sh_s, sh_c);
      }
      while (nmax < nel && guard++ < 400) {
        up = 2.0 * (up - lo) + lo;
        nmax = electron_count(n, eig, up, beta, sh_s, sh_c);
      }
      ef = 0.5 * (up + lo);
      double ne = electron_count(n, eig, ef, beta, sh_s, sh_c);
      int it = 0;
      while (fabs(nel - ne) > kElecTol && fabs(up - lo) >= fmax(fabs(ef) * eps2, eps2) && it++ < 2000) {
        if ((nmax >= nmin) == (nel >= ne)) { lo = ef; nmin = ne; }
        else { up = ef; nmax = ne; }
        ef = 0.5 * (up + lo);
        ne = electron_count(n, eig, ef, beta, sh_s, sh_c);
      }
      if (fabs(nel - ne) > kElecTolMax) status = kDevFermiFail;
      ne = electron_count(n, eig, ef, beta, sh_s, sh_c);
      if (nel > eps2 && fabs(nel - ne) > eps2) { rescale = true; ne_final = ne; }
    }
  }
  // fillings; levels after the first with f <= elecTol are zero (etemp.F90 lpLevels exit)
  if (threadIdx.x == 0) sh_i = n;
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double x = (eig[j] - ef) * beta;
    double f = 1.0 / (1.0 + exp(x));
    if (f <= kElecTol) atomicMin(&sh_i, j);
  }
  __syncthreads();
  const int j0 = sh_i;  // last level kept (inclusive)
  Comp cb = {0.0, 0.0}, ct = {0.0, 0.0};
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double f = 0.0;
    if (j <= j0) {
      double x = (eig[j] - ef) * beta;
      f = 1.0 / (1.0 + exp(x));
      if (f > kEps && f < 1.0 - kEps) neumaier(ct, -(f * log(f) + (1.0 - f) * log(1.0 - f)));
      neumaier(cb, f * eig[j]);
    }
    if (rescale) f = f * nel / ne_final;
    fill[j] = 2.0 * f;
  }
  double eb = block_csum(cb, sh_s, sh_c);
  double ts = block_csum(ct, sh_s, sh_c) * kT;
  // number of levels with |f| >= eps
  if (threadIdx.x == 0) sh_i = 0;
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    if (fabs(fill[j]) >= kEps) atomicMax(&sh_i, j + 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    scal[kSEf] = ef;
    scal[kSEband] = 2.0 * eb;
    scal[kSTS] = 2.0 * ts;
    scal[kSE0] = 2.0 * (eb - 0.5 * ts);
    scal[kSNLevels] = (double)sh_i;
    scal[kSFermiStatus] = (double)status;
  }
}

void fermi_filling(cudaStream_t s, int n, const double *eig, double nel, double kT, double *fill,
                   double *scal) {
  fermi_kernel<<<1, 1024, 0, s>>>(n, eig, nel, kT, fill, scal);
  count_launch();
}

// ------------------------------------------------------------------------------ Mulliken
// q_mu = sum_nu rho_mu,nu S_mu,nu (populations.F90:120-191), e_mu = sum_nu rho H0 (the same routine on
// H0 gives E_nonSCC, getenergies.F90:198-199). Column mu of the symmetric matrices per CTA.
__global__ void mulliken_col_kernel(int n, const double *rho, const double *S, const double *H0,
                                    double *qorb, double *eorb) {
  __shared__ double sh[2][8];
  int mu = blockIdx.x;
  const double *r = rho + (size_t)mu * n, *s = S + (size_t)mu * n, *h = H0 + (size_t)mu * n;
  double q = 0.0, e = 0.0;
  for (int nu = threadIdx.x; nu < n; nu += blockDim.x) {
    double rv = r[nu];
    q = fma(rv, s[nu], q);
    e = fma(rv, h[nu], e);
  }
  q = warp_sum(q);
  e = warp_sum(e);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sh[0][w] = q; sh[1][w] = e; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { a += sh[0][k]; b += sh[1][k]; }
    qorb[mu] = a;
    eorb[mu] = b;
  }
}

__global__ void __launch_bounds__(1024) mulliken_atom_kernel(GeomDev g, const double *qorb, const double *eorb,
                                                             double *qatom, double *scal) {
  __shared__ double sh_s[33], sh_c[33];
  for (int a = threadIdx.x; a < g.natom; a += blockDim.x) {
    double s = 0.0;
    for (int o = g.orb_off[a]; o < g.orb_off[a + 1]; ++o) s += qorb[o];
    qatom[a] = s;
  }
  Comp c = {0.0, 0.0};
  for (int o = threadIdx.x; o < g.norb; o += blockDim.x) neumaier(c, eorb[o]);
  double e = block_csum(c, sh_s, sh_c);
  if (threadIdx.x == 0) scal[kSEnonScc] = e;
}

void mulliken(cudaStream_t s, const GeomDev &g, const double *rho, const double *S, const double *H0,
              double *qorb, double *qatom, double *eorb, double *scal) {
  mulliken_col_kernel<<<g.norb, 256, 0, s>>>(g.norb, rho, S, H0, qorb, eorb);
  mulliken_atom_kernel<<<1, 1024, 0, s>>>(g, qorb, eorb, qatom, scal);
  count_launch(2);
}

__global__ void __launch_bounds__(1024) scc_energy_kernel(int natom, const double *V, const double *q,
                                                          const double *q0, double *scal) {
  __shared__ double sh_s[33], sh_c[33];
  Comp c = {0.0, 0.0};
  for (int a = threadIdx.x; a < natom; a += blockDim.x) neumaier(c, V[a] * (q[a] - q0[a]));
  double e = block_csum(c, sh_s, sh_c);
  if (threadIdx.x == 0) scal[kSEscc] = 0.5 * e;
}

void scc_energy(cudaStream_t s, int natom, const double *V, const double *q, const double *q0, double *scal) {
  scc_energy_kernel<<<1, 1024, 0, s>>>(natom, V, q, q0, scal);
  count_launch();
}

// ------------------------------------------------------------------------------ repulsive
__global__ void rep_energy_kernel(ModelDev M, GeomDev g, double *eatom) {
  int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (a >= g.natom) return;
  const int sa = g.species[a];
  double s = 0.0;
  for (int b = lane; b < g.natom; b += 32) {
    if (b == a) continue;
    double dx = g.xyz[3 * a] - g.xyz[3 * b], dy = g.xyz[3 * a + 1] - g.xyz[3 * b + 1],
           dz = g.xyz[3 * a + 2] - g.xyz[3 * b + 2];
    const PairDev &P = M.pair[g.species[b] * M.nsp + sa];
    double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 > P.rep_cut * P.rep_cut) continue;
    double e, de;
    spline_rep(M.rep + P.off_rep, P.n_spline, sqrt(r2), &e, &de);
    s += 0.5 * e;
  }
  s = warp_sum(s);
  if (lane == 0) eatom[a] = s;
}

__global__ void __launch_bounds__(1024) sum_to_scalar_kernel(int n, const double *v, double *out) {
  __shared__ double sh_s[33], sh_c[33];
  Comp c = {0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) neumaier(c, v[i]);
  double e = block_csum(c, sh_s, sh_c);
  if (threadIdx.x == 0) *out = e;
}

void repulsive_energy(cudaStream_t s, const ModelDev &m, const GeomDev &g, double *eatom, double *scal) {
  rep_energy_kernel<<<ceil_div((long long)g.natom * 32, 256), 256, 0, s>>>(m, g, eatom);
  sum_to_scalar_kernel<<<1, 1024, 0, s>>>(g.natom, eatom, scal + kSErep);
  count_launch(2);
}

// ------------------------------------------------------------------------------ Broyden
// mixer/broydenmixer.F90:204-342 (modified Broyden, Johnson 1988) in one CTA. The SCC convergence
// test max|q_out - q_in| < tol (main.F90:4907-4908) decides whether a mixing step is taken.
__global__ void __launch_bounds__(1024) broyden_kernel(int N, int it, int mix_it, int min_iter, int max_iter_scc,
                                                       double tol,
                                                       double alpha, double omega0, double minw, double maxw,
                                                       double wfac, BroydenDev B, double *qin,
                                                       const double *qout, double *scal) {
  extern __shared__ double smem[];
  __shared__ double red[33];
  __shared__ double sc[8];
  const int t = threadIdx.x;
  // error
  double mx = 0.0;
  for (int i = t; i < N; i += blockDim.x) mx = fmax(mx, fabs(qout[i] - qin[i]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((t & 31) == 0) red[t >> 5] = mx;
  __syncthreads();
  if (t == 0) {
    double m = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) m = fmax(m, red[k]);
    sc[0] = m;
  }
  __syncthreads();
  const double err = sc[0];
  const bool conv = (err < tol) && (it >= min_iter);
  if (t == 0) {
    scal[kSErr] = err;
    scal[kSConv] = conv ? 1.0 : 0.0;
  }
  if (conv || it == max_iter_scc) return;
  const int nn = mix_it;  // number of this mixing step (the mixer's own counter)
  if (nn > B.max_iter) return;
  auto bsum = [&](double v) -> double {
    v = warp_sum(v);
    __syncthreads();
    if ((t & 31) == 0) red[t >> 5] = v;
    __syncthreads();
    if (t == 0) {
      double a = 0.0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) a += red[k];
      red[32] = a;
    }
    __syncthreads();
    return red[32];
  };
  if (nn == 1) {
    for (int i = t; i < N; i += blockDim.x) {
      double d = qout[i] - qin[i];
      B.qlast[i] = qin[i];
      B.dlast[i] = d;
      qin[i] = qin[i] + alpha * d;
    }
    return;
  }
  const int n1 = nn - 1;
  const int M = B.max_iter;
  // weight
  double ss = 0.0;
  for (int i = t; i < N; i += blockDim.x) { double d = qout[i] - qin[i]; ss = fma(d, d, ss); }
  double wn = sqrt(bsum(ss));
  double ww = (wn > wfac / maxw) ? wfac / wn : maxw;
  if (ww < minw) ww = minw;
  if (t == 0) B.ww[n1 - 1] = ww;
  // df = (diff - dlast) / ||.||
  double s2 = 0.0;
  for (int i = t; i < N; i += blockDim.x) { double v = (qout[i] - qin[i]) - B.dlast[i]; s2 = fma(v, v, s2); }
  double nrm = fmax(sqrt(bsum(s2)), kEps);
  double inv = 1.0 / nrm;
  double *df = B.dF + (size_t)(n1 - 1) * N;
  for (int i = t; i < N; i += blockDim.x) df[i] = inv * ((qout[i] - qin[i]) - B.dlast[i]);
  __syncthreads();
  double *cc = smem;                 // [n1]
  double *beta = smem + M;           // [n1 x n1]
  for (int i = 0; i < n1 - 1; ++i) {
    const double *dfi = B.dF + (size_t)i * N;
    double a = 0.0, c = 0.0;
    for (int k = t; k < N; k += blockDim.x) {
      a = fma(dfi[k], df[k], a);
      c = fma(dfi[k], qout[k] - qin[k], c);
    }
    a = bsum(a);
    c = bsum(c);
    if (t == 0) {
      B.aa[i + (size_t)(n1 - 1) * M] = a;
      B.aa[(n1 - 1) + (size_t)i * M] = a;
      cc[i] = B.ww[i] * c;
    }
  }
  {
    double c = 0.0;
    for (int k = t; k < N; k += blockDim.x) c = fma(df[k], qout[k] - qin[k], c);
    c = bsum(c);
    if (t == 0) {
      B.aa[(n1 - 1) + (size_t)(n1 - 1) * M] = 1.0;
      cc[n1 - 1] = ww * c;
    }
  }
  __syncthreads();
  for (int idx = t; idx < n1 * n1; idx += blockDim.x) {
    int i = idx % n1, j = idx / n1;
    double v = B.ww[i] * B.ww[j] * B.aa[i + (size_t)j * M];
    if (i == j) v += omega0 * omega0;
    beta[i + j * n1] = v;
  }
  __syncthreads();
  // Gaussian elimination with partial pivoting on beta x = cc (beta symmetric)
  __shared__ int piv;
  for (int k = 0; k < n1; ++k) {
    if (t == 0) {
      int p = k;
      double best = fabs(beta[k + k * n1]);
      for (int i = k + 1; i < n1; ++i)
        if (fabs(beta[i + k * n1]) > best) { best = fabs(beta[i + k * n1]); p = i; }
      piv = p;
    }
    __syncthreads();
    int p = piv;
    if (p != k) {
      for (int j = t; j < n1; j += blockDim.x) {
        double tmp = beta[k + j * n1];
        beta[k + j * n1] = beta[p + j * n1];
        beta[p + j * n1] = tmp;
      }
      if (t == 0) { double tmp = cc[k]; cc[k] = cc[p]; cc[p] = tmp; }
    }
    __syncthreads();
    double dkk = beta[k + k * n1];
    for (int idx = t; idx < (n1 - k - 1) * (n1 - k); idx += blockDim.x) {
      int i = k + 1 + idx % (n1 - k - 1);
      int j = k + idx / (n1 - k - 1);
      double lik = beta[i + k * n1] / dkk;
      if (j > k) beta[i + j * n1] -= lik * beta[k + j * n1];
    }
    __syncthreads();
    if (t == 0)
      for (int i = k + 1; i < n1; ++i) cc[i] -= beta[i + k * n1] / dkk * cc[k];
    __syncthreads();
  }
  if (t == 0) {
    for (int i = n1 - 1; i >= 0; --i) {
      double v = cc[i];
      for (int j = i + 1; j < n1; ++j) v -= beta[i + j * n1] * cc[j];
      cc[i] = v / beta[i + i * n1];
    }
  }
  __syncthreads();
  // u = alpha df + inv (qin - qlast); new qin
  double *u = B.uu + (size_t)(n1 - 1) * N;
  for (int i = t; i < N; i += blockDim.x) {
    double qi = qin[i];
    double d = qout[i] - qi;
    double ui = alpha * df[i] + inv * (qi - B.qlast[i]);
    double nq = qi + alpha * d;
    for (int k = 0; k < n1 - 1; ++k) nq -= B.ww[k] * cc[k] * B.uu[(size_t)k * N + i];
    nq -= ww * cc[n1 - 1] * ui;
    B.qlast[i] = qi;
    B.dlast[i] = d;
    u[i] = ui;
    qin[i] = nq;
  }
}

void broyden_step(cudaStream_t s, int natom, int it, int mix_it, int min_iter, int max_iter_scc, double tol,
                  double alpha, double omega0, double minw, double maxw, double wfac, BroydenDev b, double *qin,
                  const double *qout, double *scal) {
  size_t smem = sizeof(double) * ((size_t)b.max_iter + (size_t)b.max_iter * b.max_iter);
  ensure_dyn_smem((const void *)broyden_kernel, 200 * 1024);
  broyden_kernel<<<1, 1024, smem, s>>>(natom, it, mix_it, min_iter, max_iter_scc, tol, alpha, omega0, minw, maxw,
                                       wfac, b, qin, qout, scal);
  count_launch();
}

// ------------------------------------------------------------------------------ forces
// derivative_blockEuclidean (forces.F90:548-669) with the central-difference block derivatives
// of getFirstDerivFiniteDiff (nonscc.F90:428-484, delta = eps^(1/4)). One warp per atom A sums the
// contributions of all partners B (each pair evaluated from both sides: deterministic, no atomics).
__global__ void __launch_bounds__(64) grad_bands_kernel(ModelDev M, GeomDev g, const double *rho,
                                                        const double *W, const double *V, double *grad) {
  __shared__ WarpSk ws_all[2][6];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int A = blockIdx.x * 2 + w;
  if (A >= g.natom) return;
  const double delta = 1.220703125e-4;  // eps^(1/4) = 2^-13
  const size_t n = g.norb;
  double gx = 0.0, gy = 0.0, gz = 0.0;
  const int sA = g.species[A];
  for (int B = 0; B < g.natom; ++B) {
    if (B == A) continue;
    const int a1 = min(A, B), a2 = max(A, B);
    const int s1 = g.species[a1], s2 = g.species[a2];
    const double bx = g.xyz[3 * a2] - g.xyz[3 * a1];
    const double by = g.xyz[3 * a2 + 1] - g.xyz[3 * a1 + 1];
    const double bz = g.xyz[3 * a2 + 2] - g.xyz[3 * a1 + 2];
    const PairDev &P = M.pair[s1 * M.nsp + s2];
    const double r2 = bx * bx + by * by + bz * bz;
    if (r2 > P.sk_cut * P.sk_cut) continue;
    for (int k = 0; k < 3; ++k)
      for (int ii = 0; ii < 2; ++ii) {
        double v[3] = {bx, by, bz};
        v[k] -= (double)(2 * (ii + 1) - 3) * delta;  // ii=0: +delta, ii=1: -delta
        eval_blocks(M, s1, s2, v[0], v[1], v[2], ws_all[w][k * 2 + ii], lane);
      }
    const int o1 = g.orb_off[a1], o2 = g.orb_off[a2];
    const int n1 = M.sp[s1].n_orb, n2 = M.sp[s2].n_orb;
    const double vs = 0.5 * (V[a1] + V[a2]);
    const double inv2d = 1.0 / (2.0 * delta);
    double dt[3] = {0.0, 0.0, 0.0};
    for (int idx = lane; idx < n1 * n2; idx += 32) {
      int b = idx % n2, a = idx / n2;
      double rv = rho[(o2 + b) + (size_t)(o1 + a) * n];
      double wv = W[(o2 + b) + (size_t)(o1 + a) * n];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double dh = (ws_all[w][2 * k + 1].blk[0][b][a] - ws_all[w][2 * k].blk[0][b][a]) * inv2d;
        double ds = (ws_all[w][2 * k + 1].blk[1][b][a] - ws_all[w][2 * k].blk[1][b][a]) * inv2d;
        dt[k] += 2.0 * (rv * dh - wv * ds) + 2.0 * vs * ds * rv;
      }
    }
    __syncwarp();
    double sgn = (A == a1) ? 1.0 : -1.0;
    gx += sgn * warp_sum(dt[0]);
    gy += sgn * warp_sum(dt[1]);
    gz += sgn * warp_sum(dt[2]);
  }
  (void)sA;
  if (lane == 0) {
    grad[3 * A] = gx;
    grad[3 * A + 1] = gy;
    grad[3 * A + 2] = gz;
  }
}

void gradient_bands(cudaStream_t s, const ModelDev &m, const GeomDev &g, const double *rho, const double *W,
                    const double *V, double *grad) {
  grad_bands_kernel<<<ceil_div(g.natom, 2), 64, 0, s>>>(m, g, rho, W, V, grad);
  count_launch();
}

// SCC double counting (shortgamma.F90:349-411, coulomb.F90:1140-1185) + repulsive
// (twobodyrep.F90:273-332), added to grad.
__global__ void grad_dc_rep_kernel(ModelDev M, GeomDev g, const double *q, const double *q0, double *grad) {
  int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (a >= g.natom) return;
  const int sa = g.species[a];
  const double ua = M.sp[sa].hubbu;
  const double dqa = q[a] - q0[a];
  double gx = 0.0, gy = 0.0, gz = 0.0;
  for (int b = lane; b < g.natom; b += 32) {
    if (b == a) continue;
    const int sb = g.species[b];
    double dx = g.xyz[3 * a] - g.xyz[3 * b], dy = g.xyz[3 * a + 1] - g.xyz[3 * b + 1],
           dz = g.xyz[3 * a + 2] - g.xyz[3 * b + 2];
    double r2 = dx * dx + dy * dy + dz * dz;
    double r = sqrt(r2);
    double qq = dqa * (q[b] - q0[b]);
    double f = -qq / (r2 * r);  // Coulomb
    double rc = M.pair[sa * M.nsp + sb].gamma_cut;
    if (r2 <= rc * rc + kTolSameDist * kTolSameDist) f -= qq * exp_gamma_prime(r, M.sp[sb].hubbu, ua) / r;
    const PairDev &P = M.pair[sb * M.nsp + sa];
    if (r2 <= P.rep_cut * P.rep_cut) {
      double e, de;
      spline_rep(M.rep + P.off_rep, P.n_spline, r, &e, &de);
      f += de / r;
    }
    gx += f * dx;
    gy += f * dy;
    gz += f * dz;
  }
  gx = warp_sum(gx);
  gy = warp_sum(gy);
  gz = warp_sum(gz);
  if (lane == 0) {
    grad[3 * a] += gx;
    grad[3 * a + 1] += gy;
    grad[3 * a + 2] += gz;
  }
}

void gradient_dc_rep(cudaStream_t s, const ModelDev &m, const GeomDev &g, const double *q, const double *q0,
                     double *grad) {
  grad_dc_rep_kernel<<<ceil_div((long long)g.natom * 32, 256), 256, 0, s>>>(m, g, q, q0, grad);
  count_launch();
}

__global__ void energy_weights_kernel(int k, const double *fill, const double *eig, double *fe) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) fe[j] = fill[j] * eig[j];
}
void energy_weights(cudaStream_t s, int k, const double *fill, const double *eig, double *fe) {
  if (k <= 0) return;
  energy_weights_kernel<<<ceil_div(k, 256), 256, 0, s>>>(k, fill, eig, fe);
  count_launch();
}

}  // namespace dg
