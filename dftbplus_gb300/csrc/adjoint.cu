// Parameter gradients of the converged SCC energy: dE/d(SK grid values) and dE/d(Hubbard U).
//
// At SCC convergence the Mermin free energy is stationary in the density matrix (under the S
// orthonormality constraint) and in the charges, so the derivative with respect to any parameter
// theta is its explicit derivative at fixed rho, W and dq:
//   dE/dtheta = sum_pairs [2 rho o dH0/dtheta + 2 (rho V_bar - W) o dS/dtheta]
//             + 1/2 sum_AB dq_A dq_B dgamma_AB/dtheta
// (the same contraction as the force, forces.F90:548-669, with d/dR replaced by d/dtheta). H0 and S
// blocks are linear in the interpolated integrals, and every integral is linear in the table values
// (8-point Lagrange window, slakoeqgrid.F90:183-244 and interpolation.F90:182-239, including the
// 5th-order tail whose value, slope and curvature at the grid end come from the same window,
// interpolation.F90:31-67), so the adjoint is exact: per pair, c_int = sum_block G o R_int with R_int
// the block of a unit integral, scattered with the window weights.
#include "dftb_device.cuh"

namespace dg {

// Window [g0, g0 + 8) and weights w[q] with integral(r) = sum_q w[q] y[g0 + q] for a table of the
// pair P (identical for every integral and for H and S). Lane q < 8 computes w[q]. Returns false
// when r is beyond the cutoff (no dependence).
static __device__ bool table_weights(const PairDev &P, double r, int lane, int *g0, double *wq) {
  const double incr = P.dist;
  const int leng = P.rows;
  const double rmax = leng * incr + kDistFudge;
  if (r >= rmax) return false;
  const int ind = (int)floor(r / incr);
  const bool tail = ind >= leng;
  int il = tail ? leng : max(min(leng, ind + 4), 8);
  *g0 = il - 8;
  *wq = 0.0;
  if (lane < 8) {
    // Lagrange basis polynomial q of the window nodes x_j = (g0 + j + 1) incr at x
    auto lag = [&](double x) {
      double v = 1.0;
      const double xq = (double)(*g0 + lane + 1) * incr;
      for (int j = 0; j < 8; ++j) {
        if (j == lane) continue;
        const double xj = (double)(*g0 + j + 1) * incr;
        v *= (x - xj) / (xq - xj);
      }
      return v;
    };
    if (!tail) {
      *wq = lag(r);
    } else {
      // value y0 = y[leng-1], slope and curvature by +-1e-5 differences of the window interpolant
      const double xa = (double)leng * incr, h = 1e-5;
      const double lp = lag(xa + h), lm = lag(xa - h);
      const double e7 = (lane == 7) ? 1.0 : 0.0;
      const double wy0 = e7, wy1 = (lp - lm) / (2.0 * h), wy2 = (lp + lm - 2.0 * e7) / (h * h);
      const double dx = -kDistFudge;
      const double xr = (r - rmax) / dx;
      const double x3 = xr * xr * xr;
      const double a = x3 * (10.0 - 15.0 * xr + 6.0 * xr * xr);
      const double b = x3 * (-4.0 + 7.0 * xr - 3.0 * xr * xr) * dx;
      const double c = x3 * (0.5 - xr + 0.5 * xr * xr) * dx * dx;
      *wq = a * wy0 + b * wy1 + c * wy2;
    }
  }
  return true;
}

// One warp per pair (i < j) of the half neighbour list.
__global__ void __launch_bounds__(128) sk_adjoint_kernel(ModelDev M, GeomDev g, const int *pi, const int *pj,
                                                         int npairs, const double *rho, const double *W,
                                                         const double *V, double *dham, double *dover) {
  __shared__ WarpSk ws_all[4];
  __shared__ double gh[4][kMaxOrb][kMaxOrb], gs[4][kMaxOrb][kMaxOrb];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int p = blockIdx.x * 4 + w;
  if (p >= npairs) return;
  const int i = pi[p], j = pj[p];
  const int si = g.species[i], sj = g.species[j];
  const double vx = g.xyz[3 * j] - g.xyz[3 * i], vy = g.xyz[3 * j + 1] - g.xyz[3 * i + 1],
               vz = g.xyz[3 * j + 2] - g.xyz[3 * i + 2];
  const double dist = sqrt(vx * vx + vy * vy + vz * vz);
  const PairDev &P = M.pair[si * M.nsp + sj];
  int g0 = 0;
  double wq = 0.0;
  if (!table_weights(P, dist, lane, &g0, &wq)) return;   // warp-uniform
  const int oi = g.orb_off[i], oj = g.orb_off[j];
  const int ni = M.sp[si].n_orb, nj = M.sp[sj].n_orb;
  const size_t n = g.norb;
  const double vs = 0.5 * (V[i] + V[j]);
  for (int idx = lane; idx < ni * nj; idx += 32) {
    const int b = idx % nj, a = idx / nj;
    const double rv = rho[(oj + b) + (size_t)(oi + a) * n];
    const double wv = W[(oj + b) + (size_t)(oi + a) * n];
    gh[w][b][a] = 2.0 * rv;
    gs[w][b][a] = 2.0 * (rv * vs - wv);
  }
  __syncwarp();
  const double l = vx / dist, m = vy / dist, nn = vz / dist;
  WarpSk &ws = ws_all[w];
  for (int k = 0; k < P.n_int; ++k) {
    if (lane < kMaxInt) {
      ws.sk[0][lane] = (lane == k) ? 1.0 : 0.0;
      ws.sk[1][lane] = (lane == k) ? 1.0 : 0.0;
    }
    __syncwarp();
    rotate_blocks(M, si, sj, l, m, nn, ws, lane);
    double ch = 0.0, cs = 0.0;
    for (int idx = lane; idx < ni * nj; idx += 32) {
      const int b = idx % nj, a = idx / nj;
      ch = fma(gh[w][b][a], ws.blk[0][b][a], ch);
      cs = fma(gs[w][b][a], ws.blk[1][b][a], cs);
    }
    ch = warp_sum(ch);
    cs = warp_sum(cs);
    if (lane < 8) {
      const size_t o = (size_t)P.off_ham + (size_t)k * P.rows + g0 + lane;
      atomicAdd(dham + o, ch * wq);
      atomicAdd(dover + o, cs * wq);
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------------------ Hubbard U
// Forward-mode dual numbers for the short-range gamma (value, derivative).
struct Dual {
  double v, d;
};
static __device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
static __device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
static __device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
static __device__ __forceinline__ Dual operator*(double s, Dual a) { return {s * a.v, s * a.d}; }
static __device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
static __device__ __forceinline__ Dual dexp(Dual a) {
  const double e = exp(a.v);
  return {e, e * a.d};
}

// shortgammafuncs.F90:97-205 (expGamma) in dual arithmetic, same branches as exp_gamma for r > 0.
static __device__ Dual gamma_sub_d(double r, Dual t1, Dual t2) {
  const Dual t12 = t1 * t1 - t2 * t2;
  const Dual t22 = t2 * t2, t24 = t22 * t22;
  const Dual rr = {r, 0.0};
  return dexp(-r * t1) * ((0.5 * (t24 * t1)) / (t12 * t12) - (t24 * t22 - 3.0 * (t24 * t1 * t1)) / (rr * t12 * t12 * t12));
}
static __device__ Dual exp_gamma_d(double r, Dual ua, Dual ub) {
  const Dual ta = 3.2 * ua, tb = 3.2 * ub;
  if (fabs(ua.v - ub.v) < kMinHubDiff) {
    const Dual tm = 0.5 * (ta + tb);
    const Dual one_r = {1.0 / r, 0.0};
    return dexp(-r * tm) * (one_r + 0.6875 * tm + (0.1875 * r) * (tm * tm) +
                            (0.02083333333333333333 * r * r) * (tm * tm * tm));
  }
  return gamma_sub_d(r, ta, tb) + gamma_sub_d(r, tb, ta);
}

// dE/dU_s = 1/2 sum_{A in s} dq_A^2 - 1/2 sum_{A != B, r <= rc} dq_A dq_B d gamma_short(r_AB)/dU_s,
// with gamma_short(r, U_B, U_A) as in the potential (coulomb 1/r does not depend on U). One warp
// per atom A; its partners B in lanes.
__global__ void hubbard_adjoint_kernel(ModelDev M, GeomDev g, const double *q, const double *q0, double *dU) {
  const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (a >= g.natom) return;
  const int sa = g.species[a];
  const double ua = M.sp[sa].hubbu;
  const double dqa = q[a] - q0[a];
  double own = (lane == 0) ? 0.5 * dqa * dqa : 0.0;   // on-site gamma_AA = U_A
  for (int b = lane; b < g.natom; b += 32) {
    if (b == a) continue;
    const int sb = g.species[b];
    const double dx = g.xyz[3 * a] - g.xyz[3 * b], dy = g.xyz[3 * a + 1] - g.xyz[3 * b + 1],
                 dz = g.xyz[3 * a + 2] - g.xyz[3 * b + 2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double rc = M.pair[sa * M.nsp + sb].gamma_cut;
    if (r2 > rc * rc + kTolSameDist * kTolSameDist) continue;
    const double r = sqrt(r2);
    const double ub = M.sp[sb].hubbu;
    const double pre = -0.5 * dqa * (q[b] - q0[b]);
    // derivative with respect to U of atom A's species (second argument) and of atom B's species
    const Dual da = exp_gamma_d(r, Dual{ub, 0.0}, Dual{ua, 1.0});
    const Dual db = exp_gamma_d(r, Dual{ub, 1.0}, Dual{ua, 0.0});
    own += pre * da.d;
    atomicAdd(dU + sb, pre * db.d);
  }
  own = warp_sum(own);
  if (lane == 0) atomicAdd(dU + sa, own);
}

void sk_adjoint(cudaStream_t s, const ModelDev &m, const GeomDev &g, const int *pi, const int *pj, int npairs,
                const double *rho, const double *W, const double *V, double *dham, double *dover) {
  if (npairs <= 0) return;
  sk_adjoint_kernel<<<ceil_div(npairs, 4), 128, 0, s>>>(m, g, pi, pj, npairs, rho, W, V, dham, dover);
  count_launch();
}

void hubbard_adjoint(cudaStream_t s, const ModelDev &m, const GeomDev &g, const double *q, const double *q0,
                     double *dU) {
  hubbard_adjoint_kernel<<<ceil_div((long long)g.natom * 32, 256), 256, 0, s>>>(m, g, q, q0, dU);
  count_launch();
}

}  // namespace dg
