// jne_accum_f64.cu -- plain FP64 fused accumulation: one warp per run.
//
// Replaces, per run, the work of rng_matrix.rs:57-141 (Gaussian path),
// johansen_statistics.rs:102-197 (F construction) and the two
// sum_of_outer_products calls of johansen_statistics.rs:32-33: instead of
// materialising B and F, each run accumulates in FP64 exactly the raw moments
// its model needs (listed in a per-(model, dim) entry table), from which the
// finalize kernel rebuilds S11 and S10.
//
// Per 32-step tile: lane t draws the increments of column t0+t (Philox), the
// first d lanes run the FP64 walk along time, and every lane adds its <= MAXE
// table entries sum_t v_t[a] * v_t[b] over the tile, where
// v_t = [W_0..W_{d-1}, z_0..z_{d-1}, 1, y, y^2, 0].  Nothing T-sized touches HBM.
#include "jne_common.cuh"
#include "jne_kernels.h"

namespace {

constexpr int kF64Warps = 4;  // warps per block

template <int MAXE, bool EXT>
__global__ void __launch_bounds__(kF64Warps * JNE_WARP)
    k_accum_f64(const jne_accum_args a, const int4* __restrict__ ent, const int nent) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int d = a.dim, T = a.steps;
  const int VS = 2 * d + 5;  // odd row stride: conflict-free column writes
  const int ZERO = 2 * d + 3;
  double* v = smem + (size_t)wib * JNE_WARP * VS;
  for (int e = lane; e < JNE_WARP * VS; e += JNE_WARP) v[e] = 0.0;

  int opA[MAXE], opB[MAXE], slot[MAXE];
#pragma unroll
  for (int m = 0; m < MAXE; m++) {
    const int e = lane + JNE_WARP * m;
    if (e < nent) {
      const int4 t = ent[e];
      opA[m] = t.x; opB[m] = t.y; slot[m] = t.z;
    } else {
      opA[m] = ZERO; opB[m] = ZERO; slot[m] = -1;
    }
  }
  const double invT = 1.0 / (double)T;
  const int nq = (d + 3) >> 2;
  const jne_round_keys rk = jne_make_round_keys(a.key0, a.key1);
  const int nwarps = gridDim.x * kF64Warps;
  __syncwarp();

  for (int run = blockIdx.x * kF64Warps + wib; run < a.n_runs; run += nwarps) {
    const uint32_t seed = a.seed_first + (uint32_t)run;
    double acc[MAXE];
#pragma unroll
    for (int m = 0; m < MAXE; m++) acc[m] = 0.0;
    double carry = 0.0;  // lane f < d: W_f at the tile start

    for (int t0 = 0; t0 < T; t0 += JNE_WARP) {
      const int i = t0 + lane;  // column i draws step s = i + 1
      const bool valid = i < T;
      double* vr = v + lane * VS;
      if (EXT) {
        const double* src = a.ext + ((size_t)run * T + (valid ? i : 0)) * d;
        for (int f = 0; f < d; f++) vr[d + f] = valid ? src[f] : 0.0;
      } else {
        for (int j = 0; j < nq; j++) {
          float z[4];
          jne_normal_quad((uint32_t)(i + 1), (uint32_t)j, seed, rk, z);
#pragma unroll
          for (int e = 0; e < 4; e++) {
            const int f = 4 * j + e;
            if (f < d) vr[d + f] = valid ? (double)z[e] : 0.0;
          }
        }
      }
      const double y = (double)(i + 1) * invT;
      vr[2 * d] = valid ? 1.0 : 0.0;
      vr[2 * d + 1] = valid ? y : 0.0;
      vr[2 * d + 2] = valid ? y * y : 0.0;
      __syncwarp();
      if (lane < d) {  // exclusive walk W_i = sum_{s <= i} z_s along the tile
        const int nv = min(JNE_WARP, T - t0);
        double W = carry;
        for (int tau = 0; tau < JNE_WARP; tau++) {
          double* vt = v + tau * VS;
          vt[lane] = tau < nv ? W : 0.0;
          W += vt[d + lane];
        }
        carry = W;
      }
      __syncwarp();
      for (int tau = 0; tau < JNE_WARP; tau++) {
        const double* vt = v + tau * VS;
#pragma unroll
        for (int m = 0; m < MAXE; m++) acc[m] = fma(vt[opA[m]], vt[opB[m]], acc[m]);
      }
      __syncwarp();
    }
#pragma unroll
    for (int m = 0; m < MAXE; m++)
      if (slot[m] >= 0) a.mom[(size_t)slot[m] * a.mom_ld + run] = acc[m];
    if (lane < d) a.mom[(size_t)jne_slot_Nz1(lane, d) * a.mom_ld + run] = carry;
  }
}

template <int MAXE>
cudaError_t launch_maxe(const jne_accum_args& a, const int4* ent, int nent, int sms, cudaStream_t st) {
  const int VS = 2 * a.dim + 5;
  const size_t shm = (size_t)kF64Warps * JNE_WARP * VS * sizeof(double);
  const int threads = kF64Warps * JNE_WARP;
  auto k = a.ext ? k_accum_f64<MAXE, true> : k_accum_f64<MAXE, false>;
  // persistent grid: the resident blocks, so every warp strides over the same number of runs
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, shm) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int needed = (a.n_runs + kF64Warps - 1) / kF64Warps;
  const int grid = needed < per_sm * sms ? needed : per_sm * sms;
  k<<<grid, threads, shm, st>>>(a, ent, nent);
  return cudaGetLastError();
}

}  // namespace

cudaError_t jne_launch_accum_f64(const jne_accum_args& a, const int4* ent, int nent, int sms, cudaStream_t st) {
  if (a.n_runs <= 0) return cudaSuccess;
  switch ((nent + JNE_WARP - 1) / JNE_WARP) {
    case 1: return launch_maxe<1>(a, ent, nent, sms, st);
    case 2: return launch_maxe<2>(a, ent, nent, sms, st);
    case 3: return launch_maxe<3>(a, ent, nent, sms, st);
    case 4: return launch_maxe<4>(a, ent, nent, sms, st);
    case 5: return launch_maxe<5>(a, ent, nent, sms, st);
    case 6: return launch_maxe<6>(a, ent, nent, sms, st);
    case 7: return launch_maxe<7>(a, ent, nent, sms, st);
    case 8: return launch_maxe<8>(a, ent, nent, sms, st);
    case 9: return launch_maxe<9>(a, ent, nent, sms, st);
    default: return cudaErrorInvalidValue;
  }
}

// Entry table of a (model, dim) pair; model < 0 requests the union of all
// five models (every slot except Nz1, which comes from the walk's end point).
int jne_build_f64_entries(int model, int d, int4* out, int cap) {
  const int W = 0, Z = d, ONE = 2 * d, Y = 2 * d + 1, YY = 2 * d + 2;
  const bool all = model < 0;
  const int nb = (!all && (model == 2 || model == 4)) ? d - 1 : d;  // walk rows entering F
  const bool need_w1 = all || model >= 1;
  const bool need_y = all || model >= 2;
  const bool need_yy = all || model == 4;
  int n = 0;
  auto put = [&](int x, int y, int s) {
    if (n < cap) out[n] = make_int4(x, y, s, 0);
    n++;
  };
  for (int p = 0; p < nb; p++)
    for (int q = p; q < nb; q++) put(W + p, W + q, jne_slot_MWW(p, q, d));
  for (int p = 0; p < nb; p++) {
    if (need_w1) put(W + p, ONE, jne_slot_MW1(p, d));
    if (need_y) put(W + p, Y, jne_slot_MWy(p, d));
    if (need_yy) put(W + p, YY, jne_slot_MWyy(p, d));
  }
  for (int a = 0; a < d; a++)
    for (int b = 0; b < nb; b++) put(Z + a, W + b, jne_slot_NzW(a, b, d));
  for (int a = 0; a < d; a++) {
    if (need_y) put(Z + a, Y, jne_slot_Nzy(a, d));
    if (need_yy) put(Z + a, YY, jne_slot_Nzyy(a, d));
  }
  return n;
}
