// Adjoint of the HFBS solve (src/hfbs.cu:586-743) with respect to the target
// and the confidence, for sm_103a.
//
// Bins, splat counts and the bistochastized normalisation depend on neither
// input, so the solve is differentiated with them fixed.  The heavy-ball
// step's Huber clamp enters by its mask (|grad| < 1.345), the invA floor
// (diag <= 1e-3) by a zero derivative.  Last to first:
//   slice^T   gz = sum over pixels of gout * w * count / den at each in-grid
//             corner (a pixel with den = 0 contributes nothing);
//   step^T    u = gh - alpha*gz; gg = mask*u; gh = beta*u;
//             gb -= invA*gg; ginvA -= (b + lambda*norm*d)*gg;
//             gz += gg - lambda*norm*N(norm*invA*gg)   (N: six-neighbour sum,
//             symmetric with the zero boundary);
//   InitZ^T   z0 = blur_b / (blur_c + 1e-7);
//   blur^T    the X -> Y -> Z Laplace blur is symmetric: the same blur;
//   invA^T    dinvA/dcsum = -invA^2 where diag > 1e-3;
//   splat^T   b = S(c*t), csum = S(c): gt = c*gb[bin], gc = t*gb[bin] + gcsum[bin]
//             (pixels in the overflow luma bin get 0).
// The step adjoint needs the forward iterate z_k of each step: kept by the
// forward (segment 1) or recomputed from checkpoints of (z, h) every S steps.
#include <algorithm>
#include <cuda_bf16.h>

#include "../../include/dtsgb.h"
#include "dtsgb_internal.cuh"
#include "hfbs_internal.cuh"

namespace dtsgb {

namespace {

constexpr int kA = 256;

__device__ __forceinline__ float ld_store(const float* p) { return *p; }
__device__ __forceinline__ float ld_store(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// slice^T, pass 1: the per-pixel scale gout / den of the forward slice
// (den = sum of the eight corners' trilinear weight * count, the overflow
// plane's counts included; 0 where den = 0), into sp (pixel layout).
__global__ void k_hb_slice_scale(const HInst* __restrict__ insts,
                                 const uchar4* __restrict__ guide,
                                 const float* __restrict__ count, const float* __restrict__ ovf,
                                 const float* __restrict__ gout, float* __restrict__ sp,
                                 HParams p) {
  const HInst I = insts[blockIdx.y];
  const long long np = (long long)I.w * I.h;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < np;
       k += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(k / I.w), x = (int)(k - (long long)y * I.w);
    const long long pix = I.pix_off + (long long)y * I.pitch + x;
    const float g = gout[pix];
    float r = 0.f;
    if (g != 0.f) {
      const float fx = (float)x * 1.0f / p.sigma_x;
      const float fy = (float)y * 1.0f / p.sigma_y;
      const float fz = (float)guide[pix].x * 1.0f / p.sigma_l;
      const float x0 = floorf(fx), y0 = floorf(fy), z0 = floorf(fz);
      const float wx = fx - x0, wy = fy - y0, wz = fz - z0;
      const int ix = (int)x0, iy = (int)y0, iz = (int)z0;
      float den = 0.f;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
        const int jx = ix + dx, jy = iy + dy, jz = iz + dz;
        float cn = 0.f;
        if (jx < I.gx && jy < I.gy) {
          if (jz < I.gl)
            cn = count[I.grid_off + ((long long)jz * I.gy + jy) * I.px + jx];
          else if (jz == I.gl)
            cn = ovf[I.plane_off + (long long)jy * I.gx + jx];  // 0 unless stored
        }
        den += (dx ? wx : 1.f - wx) * (dy ? wy : 1.f - wy) * (dz ? wz : 1.f - wz) * cn;
      }
      if (den != 0.f) r = g / den;
    }
    sp[pix] = r;
  }
}

// slice^T, pass 2: gz(ix, iy, l) = count * sum over the pixels of cells
// ix-1..ix, iy-1..iy of sp * (x weight) * (y weight) * (l weight).  Four
// threads per (ix, iy) column, one per source cell, each gathering its
// cell's pixels in a fixed order (loads issued eight pixels ahead) into its
// own level histogram in shared memory (hist[level * kGatherThreads +
// thread]); the column's first thread then adds the four histograms in
// cell order.  No atomics: bitwise-reproducible gradients.
constexpr int kGatherCols = 32;
constexpr int kGatherThreads = 4 * kGatherCols;

__global__ void __launch_bounds__(kGatherThreads)
    k_hb_slice_gather(const HInst* __restrict__ insts, const uchar4* __restrict__ guide,
                      const float* __restrict__ sp, const float* __restrict__ count,
                      float* __restrict__ gz, HParams p) {
  extern __shared__ float hist[];  // (gl + 2) x kGatherThreads
  const HInst I = insts[blockIdx.y];
  const int col = blockIdx.x * kGatherCols + (threadIdx.x >> 2), q = threadIdx.x & 3;
  const bool live = col < I.gx * I.gy;
  const int iy = live ? col / I.gx : 0, ix = live ? col - iy * I.gx : 0;
  float* hcol = hist + threadIdx.x;
  for (int l = 0; l < I.gl + 2; ++l) hcol[l * kGatherThreads] = 0.f;
  const int cx = ix - 1 + (q & 1), cy = iy - 1 + (q >> 1);  // this thread's cell
  if (live && cx >= 0 && cy >= 0) {
    const int xs = cell_start(cx, p.sigma_x, I.w), xe = cell_start(cx + 1, p.sigma_x, I.w);
    const int ys = cell_start(cy, p.sigma_y, I.h), ye = cell_start(cy + 1, p.sigma_y, I.h);
    const int nx = xe - xs, n = nx * (ye - ys);
    for (int k0 = 0; k0 < n; k0 += 8) {
      float sv[8];
      unsigned char lv[8];
      int xv[8], yv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = min(k0 + u, n - 1);
        const int dy = k / nx;
        yv[u] = ys + dy;
        xv[u] = xs + (k - dy * nx);
        const long long pix = I.pix_off + (long long)yv[u] * I.pitch + xv[u];
        sv[u] = k0 + u < n ? sp[pix] : 0.f;
        lv[u] = guide[pix].x;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (sv[u] == 0.f) continue;
        const float fx = (float)xv[u] * 1.0f / p.sigma_x;
        const float fy = (float)yv[u] * 1.0f / p.sigma_y;
        const float fx0 = floorf(fx), fy0 = floorf(fy);
        const float wxx = cx == ix ? 1.f - (fx - fx0) : fx - fx0;
        const float wyy = cy == iy ? 1.f - (fy - fy0) : fy - fy0;
        const float fz = (float)lv[u] * 1.0f / p.sigma_l;
        const float z0 = floorf(fz);
        const float wz = fz - z0;
        const int iz = (int)z0;  // <= gl
        const float a = sv[u] * wxx * wyy;
        hcol[iz * kGatherThreads] += a * (1.f - wz);
        hcol[(iz + 1) * kGatherThreads] += a * wz;
      }
    }
  }
  __syncthreads();
  if (live && q == 0) {
    for (int l = 0; l < I.gl; ++l) {
      const float* r = hcol + l * kGatherThreads;
      const float v = ((r[0] + r[1]) + r[2]) + r[3];
      const long long g = I.grid_off + ((long long)l * I.gy + iy) * I.px + ix;
      gz[g] = count[g] * v;
    }
  }
}

// step^T, one launch per step.  finish: complete the previous (later) step,
// gz += gg_in - lambda*norm*N(gw_in) (N: the six-neighbour sum; gw_in of the
// neighbours comes from the previous launch).  step: the adjoint of step k
// with its forward iterate z_k, into gh, gb, ginv and gg_out, gw_out.  The
// neighbour sum and q are formed as in the forward step (kRounded: the
// temporally blocked kernel's rounded z * n products), so the Huber mask is
// the forward's.
template <bool kRounded>
__global__ void k_hb_step_adj(const HInst* __restrict__ insts, const float* __restrict__ zk,
                              float* __restrict__ gz, float* __restrict__ gh,
                              const float* __restrict__ gg_in, const float* __restrict__ gw_in,
                              float* __restrict__ gg_out, float* __restrict__ gw_out,
                              const float* __restrict__ norm, const float* __restrict__ b,
                              const float* __restrict__ invA, float* __restrict__ gb,
                              float* __restrict__ ginv, float lambda, float alpha, float beta,
                              int finish, int step) {
  pdl_wait_then_release();  // launched as a dependent of the previous step
  const HInst I = insts[blockIdx.y];
  const int gx = I.gx, gy = I.gy, gl = I.gl;
  const long long nv = (long long)gx * gy * gl;
  const int sy = I.px, sz = I.px * gy;
  const float* nn = norm + I.grid_off;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(v / gx), x = (int)(v - (long long)r * gx);
    const int zz = r / gy, y = r - zz * gy;
    const int i = r * sy + x;  // (zz * gy + y) rows of px voxels
    const long long g = I.grid_off + i;
    float gzv = gz[g];
    const float nc = nn[i];
    if (finish) {
      const float* w = gw_in + I.grid_off;
      float a = 0.f;
      if (x > 0) a += w[i - 1];
      if (x + 1 < gx) a += w[i + 1];
      if (y > 0) a += w[i - sy];
      if (y + 1 < gy) a += w[i + sy];
      if (zz > 0) a += w[i - sz];
      if (zz + 1 < gl) a += w[i + sz];
      gzv += gg_in[g] - lambda * nc * a;
      gz[g] = gzv;
    }
    if (step) {
      const float* z = zk + I.grid_off;
      float a = 0.f;
      if (kRounded) {
        if (x > 0) a = a + __fmul_rn(z[i - 1], nn[i - 1]);
        if (x + 1 < gx) a = a + __fmul_rn(z[i + 1], nn[i + 1]);
        if (y > 0) a = a + __fmul_rn(z[i - sy], nn[i - sy]);
        if (y + 1 < gy) a = a + __fmul_rn(z[i + sy], nn[i + sy]);
        if (zz > 0) a = a + __fmul_rn(z[i - sz], nn[i - sz]);
        if (zz + 1 < gl) a = a + __fmul_rn(z[i + sz], nn[i + sz]);
      } else {
        if (x > 0) a += z[i - 1] * nn[i - 1];
        if (x + 1 < gx) a += z[i + 1] * nn[i + 1];
        if (y > 0) a += z[i - sy] * nn[i - sy];
        if (y + 1 < gy) a += z[i + sy] * nn[i + sy];
        if (zz > 0) a += z[i - sz] * nn[i - sz];
        if (zz + 1 < gl) a += z[i + sz] * nn[i + sz];
      }
      const float bc = b[g], ic = invA[g];
      const float q = (bc + lambda * nc * a) * ic;
      const float grad = z[i] - q;
      const float u = gh[g] - alpha * gzv;
      const float m = fabsf(grad) >= 1.345f ? 0.f : u;
      gh[g] = beta * u;
      gb[g] -= ic * m;
      ginv[g] -= (bc + lambda * nc * a) * m;
      gg_out[g] = m;
      gw_out[g] = nc * ic * m;
    }
  }
}

// InitZ^T: d/d blur_b into gg, d/d blur_c into gw.
__global__ void k_hb_initz_adj(const float* __restrict__ blur_c, const float* __restrict__ z0,
                               const float* __restrict__ gz, float* __restrict__ gg,
                               float* __restrict__ gw, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float e = blur_c[i] + 1e-7f;
    gg[i] = gz[i] / e;
    gw[i] = -gz[i] * z0[i] / e;
  }
}

// gb += blurred d/d blur_b; gcsum (in bc) = blurred d/d blur_c + invA^T term.
__global__ void k_hb_combine(const float* __restrict__ count, const float* __restrict__ csum,
                             const float* __restrict__ norm, const float* __restrict__ invA,
                             const float* __restrict__ bb, float* __restrict__ bc,
                             float* __restrict__ gb, const float* __restrict__ ginv,
                             float lambda, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    gb[i] += bb[i];
    const float diag = lambda * (count[i] - 2.f * norm[i] * norm[i]) + csum[i];
    if (diag > 1e-3f) bc[i] -= ginv[i] * invA[i] * invA[i];
  }
}

// splat^T into the pixel gradients.
template <typename TS>
__global__ void k_hb_splat_adj(const HInst* __restrict__ insts, const uchar4* __restrict__ guide,
                               const TS* __restrict__ target, const TS* __restrict__ conf,
                               const float* __restrict__ gb, const float* __restrict__ gcs,
                               float* __restrict__ grad_t, float* __restrict__ grad_c,
                               HParams p) {
  const HInst I = insts[blockIdx.y];
  const long long np = (long long)I.w * I.h;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < np;
       k += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(k / I.w), x = (int)(k - (long long)y * I.w);
    const long long pix = I.pix_off + (long long)y * I.pitch + x;
    const int bx = (int)floorf((float)x * 1.0f / p.sigma_x);
    const int by = (int)floorf((float)y * 1.0f / p.sigma_y);
    const int bl = (int)floorf((float)guide[pix].x * 1.0f / p.sigma_l);
    float gt = 0.f, gc = 0.f;
    if (bl < I.gl) {
      const long long g = I.grid_off + ((long long)bl * I.gy + by) * I.px + bx;
      gt = ld_store(conf + pix) * gb[g];
      gc = ld_store(target + pix) * gb[g] + gcs[g];
    }
    if (grad_t) grad_t[pix] = gt;
    if (grad_c) grad_c[pix] = gc;
  }
}

int blocks_for_n(long long n) {
  long long b = (n + kA - 1) / kA;
  if (b > 152 * 8) b = 152 * 8;
  return b < 1 ? 1 : (int)b;
}

}  // namespace

int hfbs_enqueue_backward(const HfbsBatch& B, const HParams& p, const float* gout,
                          float* grad_t, float* grad_c, cudaStream_t s) {
  const HfbsGradState& G = *B.grad;
  const int ni = B.n_inst;
  const long long tv = B.total_voxels;
  const size_t gbytes = (size_t)tv * sizeof(float);
  const float* norm = (p.bistoch_iter_max % 2) ? B.n1 : B.n0;
  const int K = p.optim_iter_max;
  const int S = G.segment;
  // z_0: hist plane 0 or checkpoint slot 0 (the z0 buffer is overwritten)
  const float* z0 = K == 0 ? B.z0 : (S == 1 ? G.hist : G.ckz);
  float* sp = grad_t ? grad_t : grad_c;
  if (!sp) return DTSGB_OK;  // no gradient asked for
  prof_begin(s, DTSGB_K_HFBS_ADJOINT);
  DTSGB_CUDA(cudaMemsetAsync(G.gz, 0, gbytes, s));
  DTSGB_CUDA(cudaMemsetAsync(G.gh, 0, gbytes, s));
  DTSGB_CUDA(cudaMemsetAsync(G.gb, 0, gbytes, s));
  DTSGB_CUDA(cudaMemsetAsync(G.ginv, 0, gbytes, s));
  const dim3 gp(blocks_for_n(B.max_pixels), ni);
  const dim3 gv(blocks_for_n(B.max_voxels), ni);
  const int gflat = blocks_for_n(tv);
  // slice^T: the per-pixel scale goes to an output plane (the last kernel
  // overwrites it)
  k_hb_slice_scale<<<gp, kA, 0, s>>>(B.d_inst, B.guide, B.count, B.ovf, gout, sp, p);
  const size_t hsmem = sizeof(float) * (size_t)(B.max_gl + 2) * kGatherThreads;
  if (hsmem > 48 * 1024)
    DTSGB_CUDA(cudaFuncSetAttribute(k_hb_slice_gather,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsmem));
  const dim3 gcol((unsigned)((B.max_cells + kGatherCols - 1) / kGatherCols), ni);
  k_hb_slice_gather<<<gcol, kGatherThreads, hsmem, s>>>(B.d_inst, B.guide, sp, B.count, G.gz,
                                                        p);
  const bool tb = hfbs_uses_tb(B);
  // (gg, gw) ping-pong: a launch reads the pair the previous one wrote
  float* pg[2] = {G.gg, G.gg2};
  float* pw[2] = {G.gw, G.gw2};
  int cur = 0, launched = 0;
  // the steps' launches are programmatic dependents of one another
  auto step_adj = [&](const float* zk) -> int {
    const int fin = launched > 0, nx = cur ^ 1;
    DTSGB_CUDA(launch_dependent(tb ? k_hb_step_adj<true> : k_hb_step_adj<false>, gv, dim3(kA),
                                0, s, B.d_inst, zk, G.gz, G.gh, pg[cur], pw[cur], pg[nx],
                                pw[nx], norm, B.b, B.invA, G.gb, G.ginv, p.lambda, p.alpha,
                                p.beta, fin, 1));
    cur = nx;
    ++launched;
    return DTSGB_OK;
  };
  if (S == 1) {
    for (int k = K - 1; k >= 0; --k)
      if (int st = step_adj(G.hist + (size_t)k * tv)) return st;
  } else {
    const int nseg = (K + S - 1) / S;
    for (int j = nseg - 1; j >= 0; --j) {
      const int start = j * S, end = std::min(K, start + S);
      auto zk = [&](int k) -> float* {
        return k == start ? G.ckz + (size_t)j * tv : G.seg + (size_t)(k - start - 1) * tv;
      };
      // recompute z_{start+1} .. z_{end-1} from the segment's checkpoint
      const float* hin = G.ckh + (size_t)j * tv;
      float* hbuf[2] = {G.hrec, G.hrec2};
      int hb = 0;
      if (!tb) {  // the one-step kernel updates h in place
        DTSGB_CUDA(cudaMemcpyAsync(G.hrec, hin, gbytes, cudaMemcpyDeviceToDevice, s));
        hin = G.hrec;
      }
      for (int k = start; k + 1 < end;) {
        const int steps = tb ? std::min(kHfbsTBSteps, end - 1 - k) : 1;
        float* hout = tb ? hbuf[hb] : G.hrec;
        hfbs_launch_steps(B, p, norm, zk(k), zk(k + steps), hin, hout, steps,
                          tb ? zk(k + 1) : nullptr, tb ? steps : 0, s);
        hin = hout;
        hb ^= 1;
        k += steps;
      }
      for (int k = end - 1; k >= start; --k)
        if (int st = step_adj(zk(k))) return st;
    }
  }
  if (launched > 0) {  // finish step 0
    k_hb_step_adj<false><<<gv, kA, 0, s>>>(B.d_inst, nullptr, G.gz, G.gh, pg[cur], pw[cur],
                                           nullptr, nullptr, norm, B.b, B.invA, G.gb, G.ginv,
                                           p.lambda, p.alpha, p.beta, 1, 0);
  }
  k_hb_initz_adj<<<gflat, kA, 0, s>>>(B.t0, z0, G.gz, G.gg, G.gw, tv);
  // blur^T of (gg, gw), gz and gh as scratch: results in t1 (for gb), t2 (gcsum)
  hfbs_launch_blur_pair(B, p, G.gg, G.gw, B.t1, B.t2, G.gz, G.gh, s);
  k_hb_combine<<<gflat, kA, 0, s>>>(B.count, B.csum, norm, B.invA, B.t1, B.t2, G.gb,
                                    G.ginv, p.lambda, tv);
  if (B.st == Storage::F32)
    k_hb_splat_adj<float><<<gp, kA, 0, s>>>(B.d_inst, B.guide, (const float*)B.target,
                                            (const float*)B.conf, G.gb, B.t2, grad_t,
                                            grad_c, p);
  else
    k_hb_splat_adj<__nv_bfloat16><<<gp, kA, 0, s>>>(
        B.d_inst, B.guide, (const __nv_bfloat16*)B.target, (const __nv_bfloat16*)B.conf,
        G.gb, B.t2, grad_t, grad_c, p);
  prof_end(s, DTSGB_K_HFBS_ADJOINT);
  DTSGB_CUDA(cudaGetLastError());
  return DTSGB_OK;
}

}  // namespace dtsgb
