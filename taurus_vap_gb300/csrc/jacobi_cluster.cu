// Block one-sided (Hestenes) Jacobi in FP32 on a thread-block cluster: the
// first stage of the canonical basis (eigenvectors of rho = V V^T).
//
// With the previous canonical basis D (or the identity), M = V^T D satisfies
// M^T M = D^T rho D; rotating column pairs of M until they are orthogonal and
// applying the same rotations to D gives the eigenvectors of rho (the column
// norms^2 are the eigenvalues).  One-sided Jacobi works on V, not on its
// square rho, so small eigenvalues keep their relative precision.
//
// The 2C column blocks (width bw = ceil(n / 2C), padded with zero columns)
// live two per CTA in a cluster of C (8, or 16 above n = 256).  A sweep is
// 2C - 1 rounds of the circle method over the blocks (block 0 fixed, the
// others move one position per round): in each round a CTA rotates all pairs
// between its two blocks (bw sub-rounds of bw disjoint pairs, one warp per
// pair), and in the first round also the pairs inside each block.  Between
// rounds the blocks move to their next CTA through distributed shared memory
// (double buffered: compute, cluster barrier, pull, cluster barrier).  The
// sweep's largest |cos| of a pair, reduced over the cluster, decides
// convergence.
//
// The hardware cluster barrier is the only wait: all CTAs of a cluster are
// co-scheduled, and every CTA takes the same number of rounds and sweeps
// (the convergence flag is read from the same cluster-wide value).
#include <cooperative_groups.h>

#include "tvap_internal.cuh"

namespace cg = cooperative_groups;

namespace tvap {

namespace {

constexpr int kJcThreads = 512;  // 16 warps: one per pair of a sub-round
constexpr int kJcMaxBw = 16;     // column pairs of a sub-round, one per warp
constexpr int kJcMaxSweeps = 30;
constexpr float kJcTol = 2.0e-6f;  // |cos| of every pair: the FP64 refinement takes it from there

// block at position p of round r (circle method over `nb` blocks, block 0
// fixed, period nb - 1)
__device__ __forceinline__ int jc_block(int r, int p, int nb) {
  const int per = nb - 1;
  return p == 0 ? 0 : 1 + ((p - 1 - r) % per + per) % per;
}

// one-sided rotation of columns a and b (M and W), one warp; returns |cos|.
// The rows stay in registers (n <= 256: at most 8 per lane) between the dot
// products and the update, the W columns are fetched while the dot products
// are reduced, and the rotation uses the fast reciprocal / reciprocal square
// root: this stage only has to reach FP32 accuracy (the FP64 refinement
// follows), and every step of the per-pair chain is latency.
template <int kJcRows>
__device__ __forceinline__ float jc_rotate(int ma, int mb, int wa, int wb, int n, int lane) {
  extern __shared__ float jc[];  // the kernel's dynamic shared memory: offsets keep the accesses in LDS/STS
  float* Ma = jc + ma;
  float* Mb = jc + mb;
  float* Wa = jc + wa;
  float* Wb = jc + wb;
  float x[kJcRows], y[kJcRows], u[kJcRows], v[kJcRows];
  float aa = 0.f, bb = 0.f, ab = 0.f;
#pragma unroll
  for (int j = 0; j < kJcRows; ++j) {
    const int r = lane + 32 * j;
    const bool ok = r < n;
    x[j] = ok ? Ma[r] : 0.f;
    y[j] = ok ? Mb[r] : 0.f;
  }
#pragma unroll
  for (int j = 0; j < kJcRows; ++j) {
    const int r = lane + 32 * j;
    const bool ok = r < n;
    u[j] = ok ? Wa[r] : 0.f;
    v[j] = ok ? Wb[r] : 0.f;
  }
#pragma unroll
  for (int j = 0; j < kJcRows; ++j) {
    aa = fmaf(x[j], x[j], aa);
    bb = fmaf(y[j], y[j], bb);
    ab = fmaf(x[j], y[j], ab);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    aa += __shfl_xor_sync(0xffffffffu, aa, off);
    bb += __shfl_xor_sync(0xffffffffu, bb, off);
    ab += __shfl_xor_sync(0xffffffffu, ab, off);
  }
  if (!(aa > 0.f && bb > 0.f) || ab == 0.f) return 0.f;
  const float cosab = fabsf(ab) * rsqrtf(aa * bb);
  if (cosab < 1.0e-8f) return cosab;
  const float zeta = __fdividef(bb - aa, 2.f * ab);
  const float az = fabsf(zeta);
  float t;
  if (az > 1.0e18f) {
    t = __fdividef(0.5f, zeta);
  } else {
    const float q = fmaf(zeta, zeta, 1.f);
    t = copysignf(__frcp_rn(az + q * rsqrtf(q)), zeta);
  }
  const float c = rsqrtf(fmaf(t, t, 1.f)), s = c * t;
#pragma unroll
  for (int j = 0; j < kJcRows; ++j) {
    const int r = lane + 32 * j;
    if (r < n) {
      Ma[r] = c * x[j] - s * y[j];
      Mb[r] = s * x[j] + c * y[j];
      Wa[r] = c * u[j] - s * v[j];
      Wb[r] = s * u[j] + c * v[j];
    }
  }
  return cosab;
}

// M64: rho = M64 M64^T columns source: column j of M = M64[j * n ..] (mt = 0)
// or row j of M64 (mt = 1, M = M64^T); W0: the basis the rotations apply to
// (identity when null); W64 receives the rotated basis.
// kJcCtas CTAs in the cluster (2 kJcCtas column blocks), kJcRows rows of a
// column per lane (n <= 32 kJcRows)
template <int kJcCtas, int kJcRows>
__global__ void __launch_bounds__(kJcThreads) jacobi_cluster_kernel(int n, const double* __restrict__ M64, int mt,
                                                                    const double* __restrict__ W0,
                                                                    double* __restrict__ W64, int* sweeps_out) {
  constexpr int kJcBlocks = 2 * kJcCtas;
  extern __shared__ float jc[];  // [buf 2][slot 2][mat 2][bw][n]
  __shared__ float wmax[kJcThreads / 32];
  __shared__ float cl_max[kJcCtas];
  cg::cluster_group cluster = cg::this_cluster();
  const int c = int(cluster.block_rank());
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int bw = (n + kJcBlocks - 1) / kJcBlocks;
  const size_t colsz = size_t(n);
  auto col = [&](int buf, int slot, int mat, int k) -> float* {
    return jc + ((size_t(buf * 2 + slot) * 2 + mat) * bw + k) * colsz;
  };
  auto off = [&](int buf, int slot, int mat, int k) -> int { return ((buf * 2 + slot) * 2 + mat) * bw * n + k * n; };
  // initial blocks: slot 0 = position c, slot 1 = position 2C - 1 - c of round 0
  for (int slot = 0; slot < 2; ++slot) {
    const int blk = jc_block(0, slot == 0 ? c : kJcBlocks - 1 - c, kJcBlocks);
    for (int idx = tid; idx < bw * n; idx += blockDim.x) {
      const int k = idx / n, r = idx - k * n;
      const int j = blk * bw + k;  // global column
      float m = 0.f, w = 0.f;
      if (j < n) {
        m = float(mt ? M64[j + size_t(r) * n] : M64[r + size_t(j) * n]);
        w = W0 ? float(W0[r + size_t(j) * n]) : (r == j ? 1.f : 0.f);
      }
      col(0, slot, 0, k)[r] = m;
      col(0, slot, 1, k)[r] = w;
    }
  }
  __syncthreads();
  int cur = 0, sweep = 0;
  for (; sweep < kJcMaxSweeps; ++sweep) {
    float mx = 0.f;
    for (int round = 0; round < kJcBlocks - 1; ++round) {
      if (round == 0) {
        // pairs inside each block: round robin over bwe = bw rounded up to
        // even (the odd one out sits out), both slots at once
        const int bwe = (bw + 1) & ~1;
        for (int sr = 0; sr < bwe - 1; ++sr) {
          const int half = bwe / 2;
          if (warp < 2 * half) {
            const int slot = warp / half, k = warp - slot * half;
            int p, q;
            if (k == 0) {
              p = sr;
              q = bwe - 1;
            } else {
              p = (sr + k) % (bwe - 1);
              q = (sr - k + (bwe - 1)) % (bwe - 1);
            }
            if (p < bw && q < bw)
              mx = fmaxf(mx, jc_rotate<kJcRows>(off(cur, slot, 0, p), off(cur, slot, 0, q), off(cur, slot, 1, p),
                                                 off(cur, slot, 1, q), n, lane));
          }
          __syncthreads();
        }
      }
      // pairs between the two blocks: sub-round sr pairs column k of slot 0
      // with column (k + sr) % bw of slot 1
      for (int sr = 0; sr < bw; ++sr) {
        if (warp < bw) {
          const int k = warp, k2 = (warp + sr) % bw;
          mx = fmaxf(mx, jc_rotate<kJcRows>(off(cur, 0, 0, k), off(cur, 1, 0, k2), off(cur, 0, 1, k),
                                             off(cur, 1, 1, k2), n, lane));
        }
        __syncthreads();
      }
      // move the blocks to their positions of the next round (after the last
      // round of a sweep too: the kJcBlocks - 1 moves of a sweep bring every
      // block back to its position of round 0)
      cluster.sync();
      const int nxt = cur ^ 1;
      // new position p pulls from old position p - 1 (1 -> kJcBlocks - 1);
      // position 0 stays
      for (int slot = 0; slot < 2; ++slot) {
        int src_cta, src_slot;
        if (slot == 0) {
          if (c == 0) {
            src_cta = 0;
            src_slot = 0;
          } else if (c == 1) {
            src_cta = 0;
            src_slot = 1;
          } else {
            src_cta = c - 1;
            src_slot = 0;
          }
        } else {
          if (c == kJcCtas - 1) {
            src_cta = c;
            src_slot = 0;
          } else {
            src_cta = c + 1;
            src_slot = 1;
          }
        }
        const float* src = cluster.map_shared_rank(col(cur, src_slot, 0, 0), src_cta);
        float* dst = col(nxt, slot, 0, 0);
        // M and W of a slot are contiguous: 2 bw n floats
        const int cnt = 2 * bw * n;
        for (int idx = tid; idx < cnt; idx += blockDim.x) dst[idx] = src[idx];
      }
      cluster.sync();
      cur = nxt;
    }
    // cluster-wide largest |cos| of the sweep
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if (lane == 0) wmax[warp] = mx;
    __syncthreads();
    if (tid == 0) {
      float m = 0.f;
      for (int w = 0; w < kJcThreads / 32; ++w) m = fmaxf(m, wmax[w]);
      float* dst = cluster.map_shared_rank(cl_max, 0);
      dst[c] = m;
    }
    cluster.sync();
    float gm = 0.f;
    {
      const float* src = cluster.map_shared_rank(cl_max, 0);
      for (int k = 0; k < kJcCtas; ++k) gm = fmaxf(gm, src[k]);
    }
    cluster.sync();  // cl_max of CTA 0 is rewritten by the next sweep
    if (gm <= kJcTol) {
      ++sweep;
      break;
    }
  }
  // after kJcBlocks - 1 rounds per sweep the blocks sit where round 0 put
  // them (the rotation period): slot s of CTA c holds block
  // jc_block(0, position)
  for (int slot = 0; slot < 2; ++slot) {
    const int blk = jc_block(0, slot == 0 ? c : kJcBlocks - 1 - c, kJcBlocks);
    for (int idx = tid; idx < bw * n; idx += blockDim.x) {
      const int k = idx / n, r = idx - k * n;
      const int j = blk * bw + k;
      if (j < n) W64[r + size_t(j) * n] = double(col(cur, slot, 1, k)[r]);
    }
  }
  if (c == 0 && tid == 0 && sweeps_out) *sweeps_out = sweep;
}

}  // namespace

namespace {

template <int CT, int ROWS>
int launch_jacobi_cluster(int n, const double* M, int m_transposed, const double* W0, double* W, int* sweeps_out,
                          cudaStream_t s) {
  const int bw = (n + 2 * CT - 1) / (2 * CT);
  if (bw > kJcMaxBw || n > 32 * ROWS) return TVAP_ERR_ARG;
  const size_t shm = sizeof(float) * 8 * size_t(bw) * n;
  if (shm > size_t(200) * 1024) return TVAP_ERR_ARG;
  auto kern = jacobi_cluster_kernel<CT, ROWS>;
  if (shm > 48 * 1024)
    if (int rc = smem_opt_in((const void*)kern, shm)) return rc;
  if (CT > 8) {
    // a cluster of more than 8 CTAs is an opt-in size; refused or not
    // schedulable here -> the caller takes another eigensolver
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      return TVAP_ERR_ARG;
    }
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CT);
  cfg.blockDim = dim3(kJcThreads);
  cfg.dynamicSmemBytes = shm;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CT;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (CT > 8) {
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, (const void*)kern, &cfg) != cudaSuccess || clusters < 1) {
      cudaGetLastError();
      return TVAP_ERR_ARG;
    }
  }
  ++g_launch_count;
  TVAP_CUDA(cudaLaunchKernelEx(&cfg, kern, n, M, m_transposed, W0, W, sweeps_out));
  return TVAP_OK;
}

}  // namespace

// FP32 block one-sided Jacobi on a cluster: 8 CTAs (16 column blocks) up to
// n = 256, 16 CTAs (32 column blocks, an opt-in cluster size) up to n = 384;
// TVAP_ERR_ARG when neither fits (the caller then uses another eigensolver).
int jacobi_cluster(int n, const double* M, int m_transposed, const double* W0, double* W, int* sweeps_out,
                   cudaStream_t s) {
  if (n <= 256) return launch_jacobi_cluster<8, 8>(n, M, m_transposed, W0, W, sweeps_out, s);
  return launch_jacobi_cluster<16, 12>(n, M, m_transposed, W0, W, sweeps_out, s);
}

}  // namespace tvap
