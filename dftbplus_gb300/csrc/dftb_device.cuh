// Device helpers shared by the single-system and the batched kernels: accuracy constants, SK
// table interpolation and rotations (diatomic H/S blocks), short-range gamma, repulsive splines,
// compensated sums. Included by each translation unit (internal linkage, no relocatable code).
#pragma once
#include "dftb_kernels.cuh"

namespace dg {

constexpr double kEps = 2.220446049250313e-16;
constexpr double kDistFudge = 1.0;           // common/accuracy.F90:44
constexpr double kElecTol = 1e-15;           // accuracy.F90:55
constexpr double kElecTolMax = 1e-7;         // accuracy.F90:61
constexpr double kTolSameDist = 1e-5;        // accuracy.F90:69
constexpr double kMinHubDiff = 0.3125e-5;    // accuracy.F90:110
constexpr double kMinNeighDist = 1e-2;       // accuracy.F90:78
constexpr double kSq3 = 1.7320508075688772935;

static __device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ------------------------------------------------------------------------------ SK integrals
// 8-point Neville on the uniform grid (math/interpolation.F90:182-239, polyInterU2) for one column.
static __device__ double neville8(const double *col, double incr, double x, int il) {
  double c[8], d[8], xp[8];
#pragma unroll
  for (int ii = 0; ii < 8; ++ii) {
    xp[ii] = (double)(il - 8 + ii + 1) * incr;
    c[ii] = d[ii] = col[il - 8 + ii];
  }
  // 1 / (xp[mm] - xp[0]) = 1 / (mm incr): one reciprocal and constant factors instead of seven
  // divisions (a division is a long FP64 sequence on this GPU)
  double delta[8];
  const double inv_incr = 1.0 / incr;
#pragma unroll
  for (int mm = 1; mm < 8; ++mm) delta[mm] = inv_incr * (1.0 / (double)mm);
  int icl = (int)ceil((x - xp[0]) * delta[1]);  // 1-based
  icl = max(1, min(8, icl));                     // only binds for r < 4 grid steps (no valid pair)
  double y = col[il - 8 + icl - 1];
  icl -= 1;
#pragma unroll
  for (int mm = 1; mm < 8; ++mm) {
#pragma unroll
    for (int i = 1; i <= 8 - mm; ++i) {
      double r2 = (d[i - 1] - c[i]) * delta[mm];
      c[i - 1] = (xp[i - 1] - x) * r2;
      d[i - 1] = (xp[i - 1 + mm] - x) * r2;
    }
    double dy;
    if (2 * icl < 8 - mm) {
      dy = 0.0;
#pragma unroll
      for (int q = 0; q < 8; ++q) if (q == icl) dy = c[q];
    } else {
      dy = 0.0;
#pragma unroll
      for (int q = 0; q < 8; ++q) if (q == icl - 1) dy = d[q];
      icl -= 1;
    }
    y += dy;
  }
  return y;
}

// Integral k of pair table at distance r (slakoeqgrid.F90:183-244): Neville inside the grid,
// 5th-order polynomial to zero over the last Bohr (poly5ToZero, interpolation.F90:31-67), 0 beyond.
static __device__ double sk_value(const PairDev &P, const double *tab, bool over, int k, double r) {
  const double incr = P.dist;
  const int leng = P.rows;
  const double rmax = leng * incr + kDistFudge;
  if (r >= rmax) return 0.0;
  int ind = (int)floor(r / incr);
  if (ind < leng) {
    int il = min(leng, ind + 4);
    il = max(il, 8);
    const double *col = tab + (over ? P.off_over : P.off_ham) + (size_t)k * leng;
    return neville8(col, incr, r, il);
  }
  const double(*tl)[kMaxInt] = over ? P.tail_s : P.tail_h;
  double y0 = tl[0][k], y0p = tl[1][k], y0pp = tl[2][k];
  double dx = -kDistFudge, invdx = -1.0 / kDistFudge;
  double dx1 = y0p * dx, dx2 = y0pp * dx * dx;
  double dd = 10.0 * y0 - 4.0 * dx1 + 0.5 * dx2;
  double ee = -15.0 * y0 + 7.0 * dx1 - 1.0 * dx2;
  double ff = 6.0 * y0 - 3.0 * dx1 + 0.5 * dx2;
  double xr = (r - rmax) * invdx;
  return ((ff * xr + ee) * xr + dd) * xr * xr * xr;
}

// ------------------------------------------------------------------------------ SK rotations
// R[b][a] = <a (shell lo) at atom 1 | b (shell hi) at atom 2> for unit vector (l, m, n) from 1 to
// 2; orbital order p = (y, z, x), d = (xy, yz, z2, xz, x2-y2) (Slater-Koster 1954 table).
static __device__ void rot_lohi(int lo, int hi, double l, double m, double n, const double *sk, double R[5][5]) {
  const double l2 = l * l, m2 = m * m, n2 = n * n;
  if (lo == 0 && hi == 0) {
    R[0][0] = sk[0];
  } else if (lo == 0 && hi == 1) {
    R[0][0] = m * sk[0]; R[1][0] = n * sk[0]; R[2][0] = l * sk[0];
  } else if (lo == 0 && hi == 2) {
    double s = sk[0];
    R[0][0] = kSq3 * l * m * s;
    R[1][0] = kSq3 * m * n * s;
    R[2][0] = (n2 - 0.5 * (l2 + m2)) * s;
    R[3][0] = kSq3 * l * n * s;
    R[4][0] = 0.5 * kSq3 * (l2 - m2) * s;
  } else if (lo == 1 && hi == 1) {
    double c[3] = {m, n, l};
    double sg = sk[0], pi = sk[1];
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) R[b][a] = c[b] * c[a] * (sg - pi) + (a == b ? pi : 0.0);
  } else if (lo == 1 && hi == 2) {
    double sg = sk[0], pi = sk[1];
    double q = n2 - 0.5 * (l2 + m2);
    // p_x column (a = 2)
    R[0][2] = kSq3 * l2 * m * sg + m * (1 - 2 * l2) * pi;
    R[1][2] = kSq3 * l * m * n * sg - 2 * l * m * n * pi;
    R[2][2] = l * q * sg - kSq3 * l * n2 * pi;
    R[3][2] = kSq3 * l2 * n * sg + n * (1 - 2 * l2) * pi;
    R[4][2] = 0.5 * kSq3 * l * (l2 - m2) * sg + l * (1 - l2 + m2) * pi;
    // p_y column (a = 0)
    R[0][0] = kSq3 * m2 * l * sg + l * (1 - 2 * m2) * pi;
    R[1][0] = kSq3 * m2 * n * sg + n * (1 - 2 * m2) * pi;
    R[2][0] = m * q * sg - kSq3 * m * n2 * pi;
    R[3][0] = kSq3 * l * m * n * sg - 2 * l * m * n * pi;
    R[4][0] = 0.5 * kSq3 * m * (l2 - m2) * sg - m * (1 + l2 - m2) * pi;
    // p_z column (a = 1)
    R[0][1] = kSq3 * l * m * n * sg - 2 * l * m * n * pi;
    R[1][1] = kSq3 * n2 * m * sg + m * (1 - 2 * n2) * pi;
    R[2][1] = n * q * sg + kSq3 * n * (l2 + m2) * pi;
    R[3][1] = kSq3 * n2 * l * sg + l * (1 - 2 * n2) * pi;
    R[4][1] = 0.5 * kSq3 * n * (l2 - m2) * sg - n * (l2 - m2) * pi;
  } else {  // d-d
    const double sg = sk[0], pi = sk[1], de = sk[2];
    const double lm2 = l2 - m2;
    const double q = n2 - 0.5 * (l2 + m2);
    enum { XY = 0, YZ = 1, Z2 = 2, XZ = 3, X2 = 4 };
    auto put = [&](int i, int j, double s, double p, double d) {
      double v = s * sg + p * pi + d * de;
      R[i][j] = v;
      R[j][i] = v;
    };
    put(XY, XY, 3 * l2 * m2, l2 + m2 - 4 * l2 * m2, n2 + l2 * m2);
    put(YZ, YZ, 3 * m2 * n2, m2 + n2 - 4 * m2 * n2, l2 + m2 * n2);
    put(XZ, XZ, 3 * n2 * l2, n2 + l2 - 4 * n2 * l2, m2 + n2 * l2);
    put(XY, YZ, 3 * l * m2 * n, l * n * (1 - 4 * m2), l * n * (m2 - 1));
    put(XY, XZ, 3 * l2 * m * n, m * n * (1 - 4 * l2), m * n * (l2 - 1));
    put(YZ, XZ, 3 * l * m * n2, l * m * (1 - 4 * n2), l * m * (n2 - 1));
    put(XY, X2, 1.5 * l * m * lm2, -2 * l * m * lm2, 0.5 * l * m * lm2);
    put(YZ, X2, 1.5 * m * n * lm2, -m * n * (1 + 2 * lm2), m * n * (1 + 0.5 * lm2));
    put(XZ, X2, 1.5 * n * l * lm2, n * l * (1 - 2 * lm2), -n * l * (1 - 0.5 * lm2));
    put(XY, Z2, kSq3 * l * m * q, -2 * kSq3 * l * m * n2, 0.5 * kSq3 * l * m * (1 + n2));
    put(YZ, Z2, kSq3 * m * n * q, kSq3 * m * n * (l2 + m2 - n2), -0.5 * kSq3 * m * n * (l2 + m2));
    put(XZ, Z2, kSq3 * l * n * q, kSq3 * l * n * (l2 + m2 - n2), -0.5 * kSq3 * l * n * (l2 + m2));
    put(X2, X2, 0.75 * lm2 * lm2, l2 + m2 - lm2 * lm2, n2 + 0.25 * lm2 * lm2);
    put(X2, Z2, 0.5 * kSq3 * lm2 * q, kSq3 * n2 * (m2 - l2), 0.25 * kSq3 * (1 + n2) * lm2);
    put(Z2, Z2, q * q, 3 * n2 * (l2 + m2), 0.75 * (l2 + m2) * (l2 + m2));
  }
}

struct WarpSk {
  double sk[2][kMaxInt];
  double blk[2][kMaxOrb][kMaxOrb];   // [H|S][row: orbital of atom 2][col: orbital of atom 1]
};

// Diatomic H and S blocks for species (sp1, sp2) and vector v = R2 - R1 (sk.F90:35-140 layout).
// Rotation of the integrals in ws.sk (H in sk[0], S in sk[1]) into the blocks ws.blk for species
// (sp1, sp2) and unit vector (l, m, n) from atom 1 to atom 2; linear in ws.sk.
static __device__ void rotate_blocks(const ModelDev &M, int sp1, int sp2, double l, double m, double n, WarpSk &ws,
                                     int lane) {
  const SpeciesDev &A = M.sp[sp1];
  const SpeciesDev &B = M.sp[sp2];
  const int npair = A.n_shell * B.n_shell;
  for (int t = lane; t < 2 * npair; t += 32) {
    int mat = t / npair, sidx = t % npair;
    int sh1 = sidx / B.n_shell, sh2 = sidx % B.n_shell;
    int ind = 0, col0 = 0, row0 = 0;
    for (int a = 0; a < A.n_shell; ++a)
      for (int b = 0; b < B.n_shell; ++b)
        if (a < sh1 || (a == sh1 && b < sh2)) ind += min(A.ang[a], B.ang[b]) + 1;
    for (int a = 0; a < sh1; ++a) col0 += 2 * A.ang[a] + 1;
    for (int b = 0; b < sh2; ++b) row0 += 2 * B.ang[b] + 1;
    const int l1 = A.ang[sh1], l2 = B.ang[sh2];
    const double *skp = &ws.sk[mat][ind];
    double R[5][5];
    if (l1 <= l2) {
      rot_lohi(l1, l2, l, m, n, skp, R);
      for (int b = 0; b < 2 * l2 + 1; ++b)
        for (int a = 0; a < 2 * l1 + 1; ++a) ws.blk[mat][row0 + b][col0 + a] = R[b][a];
    } else {
      rot_lohi(l2, l1, l, m, n, skp, R);
      const double sg = ((l1 + l2) & 1) ? -1.0 : 1.0;
      for (int b = 0; b < 2 * l2 + 1; ++b)
        for (int a = 0; a < 2 * l1 + 1; ++a) ws.blk[mat][row0 + b][col0 + a] = sg * R[a][b];
    }
  }
  __syncwarp();
}

static __device__ void eval_blocks(const ModelDev &M, int sp1, int sp2, double vx, double vy, double vz,
                                   WarpSk &ws, int lane) {
  const double dist = sqrt(vx * vx + vy * vy + vz * vz);
  const double l = vx / dist, m = vy / dist, n = vz / dist;
  const PairDev &P = M.pair[sp1 * M.nsp + sp2];
  if (lane < P.n_int) ws.sk[0][lane] = sk_value(P, M.tab, false, lane, dist);
  if (lane >= 16 && lane - 16 < P.n_int) ws.sk[1][lane - 16] = sk_value(P, M.tab, true, lane - 16, dist);
  __syncwarp();
  rotate_blocks(M, sp1, sp2, l, m, n, ws, lane);
}

// ------------------------------------------------------------------------------ short gamma
// shortgammafuncs.F90:97-205 (expGamma / expGammaPrime)
static __device__ double gamma_sub(double r, double t1, double t2) {
  double t12 = t1 * t1 - t2 * t2;
  return exp(-t1 * r) * ((0.5 * t2 * t2 * t2 * t2 * t1 / (t12 * t12)) -
                         (t2 * t2 * t2 * t2 * t2 * t2 - 3.0 * t2 * t2 * t2 * t2 * t1 * t1) / (r * t12 * t12 * t12));
}
static __device__ double gamma_sub_prime(double r, double t1, double t2) {
  double t12 = t1 * t1 - t2 * t2;
  double e = exp(-t1 * r);
  double num = t2 * t2 * t2 * t2 * t2 * t2 - 3.0 * t2 * t2 * t2 * t2 * t1 * t1;
  return -t1 * e * ((0.5 * t2 * t2 * t2 * t2 * t1 / (t12 * t12)) - num / (r * t12 * t12 * t12)) +
         e * num / (r * r * t12 * t12 * t12);
}
static __device__ double exp_gamma(double r, double ua, double ub) {
  double ta = 3.2 * ua, tb = 3.2 * ub;
  if (r < kTolSameDist) {
    if (fabs(ua - ub) < kMinHubDiff) return -0.5 * (ua + ub);
    return -0.5 * ((ta * tb) / (ta + tb) + (ta * tb) * (ta * tb) / ((ta + tb) * (ta + tb) * (ta + tb)));
  }
  if (fabs(ua - ub) < kMinHubDiff) {
    double tm = 0.5 * (ta + tb);
    return exp(-tm * r) * (1.0 / r + 0.6875 * tm + 0.1875 * r * tm * tm +
                           0.02083333333333333333 * r * r * tm * tm * tm);
  }
  return gamma_sub(r, ta, tb) + gamma_sub(r, tb, ta);
}
static __device__ double exp_gamma_prime(double r, double ua, double ub) {
  if (r < kTolSameDist) return 0.0;
  if (fabs(ua - ub) < kMinHubDiff) {
    double tm = 3.2 * 0.5 * (ua + ub);
    double e = exp(-tm * r);
    return -tm * e * (1.0 / r + 0.6875 * tm + 0.1875 * r * tm * tm + 0.02083333333333333333 * r * r * tm * tm * tm) +
           e * (-1.0 / (r * r) + 0.1875 * tm * tm + 2.0 * 0.02083333333333333333 * r * tm * tm * tm);
  }
  return gamma_sub_prime(r, 3.2 * ua, 3.2 * ub) + gamma_sub_prime(r, 3.2 * ub, 3.2 * ua);
}

struct Comp {
  double s, c;
};
static __device__ __forceinline__ void neumaier(Comp &a, double x) {
  double t = a.s + x;
  if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
  else a.c += (x - t) + a.s;
  a.s = t;
}
// dftb/repulsive/splinerep.F90:136-266
static __device__ void spline_rep(const double *rd, int nspl, double r, double *e, double *de) {
  const double cutoff = rd[0];
  const double *ec = rd + 1;
  const double *xs = rd + 4;
  const double *cub = xs + nspl;
  const double *last = cub + 4 * (nspl - 1);
  *e = 0.0;
  *de = 0.0;
  if (r < kMinNeighDist || r >= cutoff) return;
  if (r < xs[0]) {
    double ex = exp(-ec[0] * r + ec[1]);
    *e = ex + ec[2];
    *de = -ec[0] * ex;
    return;
  }
  int lo = 0, hi = nspl;
  while (lo < hi) {
    int cur = lo + (hi - lo + 1) / 2;
    if (r - xs[cur - 1] >= -kEps) lo = cur; else hi = cur - 1;
  }
  const int im = lo;  // 1-based
  const double dr = r - xs[im - 1];
  const double *k = (im < nspl) ? cub + 4 * (im - 1) : last;
  const int nk = (im < nspl) ? 4 : 6;
  double ev = k[0], xh = dr;
  for (int t = 1; t < nk; ++t) { ev += k[t] * xh; xh *= dr; }
  double dv = 0.0;
  xh = 1.0;
  for (int t = 1; t < nk; ++t) { dv += t * k[t] * xh; xh *= dr; }
  *e = ev;
  *de = dv;
}


}  // namespace dg
