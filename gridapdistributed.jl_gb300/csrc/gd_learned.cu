// Learned preconditioner for the mixed-precision flexible CG (3D Q1 spaces).
//
// An L-level (default 3), 8-channel convolutional network on the structured node
// lattice, used in a form that is symmetric positive definite by construction:
//   z = D^-1 r + D^-1/2 S^T S D^-1/2 r
// S is a coefficient-gated encoder (features at every level):
//   f_0 = log(kappa at the nodes), f_l = R f_{l-1}                 (once per problem)
//   s_l = sigmoid(conv3(f_l; G_l) + b_l)                            (8 channels, per problem)
//   x_0 = D^-1/2 r on the lattice (0 on Dirichlet nodes), x_l = R h_{l-1}
//   h_l = conv3(x_l; W_l) * s_l                                     (1->8, then 8->8)
//   S x_0 = (h_0, ..., h_{L-1})
// and S^T is its exact adjoint (the decoder shares the encoder's weights: a U-net with
// tied weights), so the learned term is positive semi-definite and plain (or flexible)
// CG applies.  With the coarse-start option the network runs on the once-restricted
// lattice, z = D^-1 r + D^-1/2 R^T S^T S R D^-1/2 r (still SPD): the fine-scale error is
// left to the Jacobi term and the costliest level of the application disappears.  R is full-weighting restriction (coarse node i <-> fine node 2i), P = 8 R^T
// trilinear prolongation, conv3 a 3x3x3 convolution with zero padding.  Training
// minimises the relative A-norm error ||z - e||_A^2 / ||e||_A^2 over (residual, error)
// pairs generated by the solver, with hand-written backward kernels and Adam.  All in
// FP32; every reduction is two-stage in a fixed order (deterministic).
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gd_internal.h"
#include "gd_solve_mixed.h"

namespace gd {

constexpr int kC = 8;          // channels
constexpr int kTaps = 27;
constexpr int kLT = 256;       // threads per block for lattice kernels
constexpr int kTile = 8;       // weight-gradient tiles are 8^3 voxels

struct Dims {
  int n[3];
  __host__ __device__ int64_t size() const { return (int64_t)n[0] * n[1] * n[2]; }
};

__host__ __device__ inline Dims coarse_dims(const Dims& f) {
  Dims c;
  for (int d = 0; d < 3; ++d) c.n[d] = f.n[d] > 1 ? (f.n[d] + 1) / 2 : 1;
  return c;
}

// ---- convolution --------------------------------------------------------------------------
// out[co][v] (+)= sum_ci sum_tap W[co][ci][tap] * in[ci][v + off(tap)], zero padding.
// mode 0: forward; mode 1: adjoint with respect to the input (W flipped and transposed).
template <int CI, int CO>
__global__ void __launch_bounds__(kLT) k_conv3(Dims d, const float* __restrict__ in, const float* __restrict__ W,
                                               const float* __restrict__ gate, const float* __restrict__ bias,
                                               float* __restrict__ out, int mode, int accumulate) {
  __shared__ float sw[CO * CI * kTaps];
  for (int i = threadIdx.x; i < CO * CI * kTaps; i += blockDim.x) {
    if (mode == 0) {
      sw[i] = W[i];
    } else {   // sw[co'][ci'][tap] = W[ci'][co'][26 - tap] for the adjoint (here CO = original CI)
      const int tap = i % kTaps, ci = (i / kTaps) % CI, co = i / (kTaps * CI);
      sw[i] = W[(ci * CO + co) * kTaps + (kTaps - 1 - tap)];
    }
  }
  __syncthreads();
  const int64_t nv = d.size();
  const int64_t plane = (int64_t)d.n[0] * d.n[1];
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(v % d.n[0]);
    const int y = (int)((v / d.n[0]) % d.n[1]);
    const int z = (int)(v / plane);
    float acc[CO];
#pragma unroll
    for (int co = 0; co < CO; ++co) acc[co] = bias ? bias[co] : 0.f;
#pragma unroll
    for (int tap = 0; tap < kTaps; ++tap) {
      const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dz = tap / 9 - 1;
      const int xx = x + dx, yy = y + dy, zz = z + dz;
      if (xx < 0 || xx >= d.n[0] || yy < 0 || yy >= d.n[1] || zz < 0 || zz >= d.n[2]) continue;
      const int64_t u = xx + (int64_t)d.n[0] * (yy + (int64_t)d.n[1] * zz);
#pragma unroll
      for (int ci = 0; ci < CI; ++ci) {
        const float val = __ldg(in + ci * nv + u);
#pragma unroll
        for (int co = 0; co < CO; ++co) acc[co] = fmaf(sw[(co * CI + ci) * kTaps + tap], val, acc[co]);
      }
    }
#pragma unroll
    for (int co = 0; co < CO; ++co) {
      float r = acc[co];
      if (gate) r *= gate[co * nv + v];
      if (accumulate) out[co * nv + v] += r;
      else out[co * nv + v] = r;
    }
  }
}

// weight gradient partials: part[tile][co][ci][tap] = sum_{v in tile} in[ci][v+off] * g[co][v]
template <int CI, int CO>
__global__ void __launch_bounds__(kLT) k_conv3_wgrad(Dims d, const float* __restrict__ in, const float* __restrict__ g,
                                                     float* __restrict__ part) {
  constexpr int H = kTile + 2;
  __shared__ float sin_[CI * H * H * H];
  __shared__ float sg[CO * kTile * kTile * kTile];
  const int tiles_x = (d.n[0] + kTile - 1) / kTile, tiles_y = (d.n[1] + kTile - 1) / kTile;
  const int t = blockIdx.x;
  const int tx = t % tiles_x, ty = (t / tiles_x) % tiles_y, tz = t / (tiles_x * tiles_y);
  const int x0 = tx * kTile, y0 = ty * kTile, z0 = tz * kTile;
  const int64_t nv = d.size();
  for (int i = threadIdx.x; i < CI * H * H * H; i += blockDim.x) {
    const int ci = i / (H * H * H), r = i % (H * H * H);
    const int hx = r % H, hy = (r / H) % H, hz = r / (H * H);
    const int xx = x0 + hx - 1, yy = y0 + hy - 1, zz = z0 + hz - 1;
    float val = 0.f;
    if (xx >= 0 && xx < d.n[0] && yy >= 0 && yy < d.n[1] && zz >= 0 && zz < d.n[2])
      val = in[ci * nv + xx + (int64_t)d.n[0] * (yy + (int64_t)d.n[1] * zz)];
    sin_[i] = val;
  }
  for (int i = threadIdx.x; i < CO * kTile * kTile * kTile; i += blockDim.x) {
    const int co = i / (kTile * kTile * kTile), r = i % (kTile * kTile * kTile);
    const int lx = r % kTile, ly = (r / kTile) % kTile, lz = r / (kTile * kTile);
    const int xx = x0 + lx, yy = y0 + ly, zz = z0 + lz;
    float val = 0.f;
    if (xx < d.n[0] && yy < d.n[1] && zz < d.n[2]) val = g[co * nv + xx + (int64_t)d.n[0] * (yy + (int64_t)d.n[1] * zz)];
    sg[i] = val;
  }
  __syncthreads();
  constexpr int NW = CO * CI * kTaps;
  for (int w = threadIdx.x; w < NW; w += blockDim.x) {
    const int tap = w % kTaps, ci = (w / kTaps) % CI, co = w / (kTaps * CI);
    const int dx = tap % 3, dy = (tap / 3) % 3, dz = tap / 9;   // halo offsets (off + 1)
    float acc = 0.f;
    for (int lz = 0; lz < kTile; ++lz)
      for (int ly = 0; ly < kTile; ++ly)
#pragma unroll
        for (int lx = 0; lx < kTile; ++lx)
          acc = fmaf(sin_[ci * H * H * H + (lx + dx) + H * ((ly + dy) + H * (lz + dz))],
                     sg[co * kTile * kTile * kTile + lx + kTile * (ly + kTile * lz)], acc);
    part[(int64_t)t * NW + w] = acc;
  }
}

// bias gradient partials: part[block][co] = sum_v g[co][v]
__global__ void k_bias_grad(Dims d, int co_n, const float* __restrict__ g, float* __restrict__ part) {
  __shared__ float sh[kLT];
  const int64_t nv = d.size();
  for (int co = 0; co < co_n; ++co) {
    float a = 0.f;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x)
      a += g[co * nv + v];
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x * co_n + co] = sh[0];
    __syncthreads();
  }
}

// out[w] (+)= sum_p part[p][w] (fixed order)
__global__ void k_sum_partials(int nparts, int nw, const float* __restrict__ part, float* __restrict__ out) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  float a = 0.f;
  for (int p = 0; p < nparts; ++p) a += part[(int64_t)p * nw + w];
  out[w] += a;
}

// load modes and epilogues of the application convolutions (described at k_tconv)
enum { LD_PLAIN = 0, LD_GATED = 1, LD_GATHER = 2 };
enum { EP_GATE = 0, EP_PLAIN = 1, EP_OUT = 2, EP_OUTLAT = 3 };

struct TConvArgsS {   // direct convolution: output channels co_n, input/gate/weights as in k_tconv
  Dims d;
  const float* in;
  const float* in_gate;
  const float* W;
  int adjoint;
  int co_n;
  const float* out_gate;
  float* out;
};

// ---- restriction / prolongation ----------------------------------------------------------
// One thread per (output voxel, channel), channel-major so a warp covers consecutive
// voxels of one channel; 32-bit index arithmetic (lattices stay below 2^31 / 8 nodes).
// coarse[ch][i] = scale * sum_{o in {-1,0,1}^3} w(o) fine[ch][2i+o], w = prod(1/2 if o=0 else 1/4)
__global__ void k_restrict(int C, Dims f, Dims c, const float* __restrict__ fine, float* __restrict__ coarse,
                           float scale) {
  const int nc = (int)c.size(), nf = (int)f.size();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < C * nc; v += gridDim.x * blockDim.x) {
    const int ch = v / nc, i = v - ch * nc;
    const int ix = i % c.n[0], iy = (i / c.n[0]) % c.n[1], iz = i / (c.n[0] * c.n[1]);
    const float* src = fine + (size_t)ch * nf;
    float acc = 0.f;
#pragma unroll
    for (int oz = -1; oz <= 1; ++oz) {
      const int fz = 2 * iz + oz;
      if (fz < 0 || fz >= f.n[2]) continue;
#pragma unroll
      for (int oy = -1; oy <= 1; ++oy) {
        const int fy = 2 * iy + oy;
        if (fy < 0 || fy >= f.n[1]) continue;
#pragma unroll
        for (int ox = -1; ox <= 1; ++ox) {
          const int fx = 2 * ix + ox;
          if (fx < 0 || fx >= f.n[0]) continue;
          const float w = (ox == 0 ? 0.5f : 0.25f) * (oy == 0 ? 0.5f : 0.25f) * (oz == 0 ? 0.5f : 0.25f);
          acc = fmaf(w, __ldg(src + fx + f.n[0] * (fy + f.n[1] * fz)), acc);
        }
      }
    }
    coarse[(size_t)ch * nc + i] = scale * acc;
  }
}

// trilinear neighbours of fine voxel j along one axis: j even -> coarse j/2 (weight 1);
// j odd -> (j-1)/2 and (j+1)/2 (weights 1/2, the second only inside the coarse lattice)
struct Lin1 {
  int i0, i1, cnt;
  float w;
};
__device__ inline Lin1 lin1(int j, int nc) {
  Lin1 r;
  if ((j & 1) == 0) {
    r.i0 = r.i1 = j >> 1;
    r.cnt = 1;
    r.w = 1.f;
  } else {
    r.i0 = j >> 1;
    r.i1 = (j >> 1) + 1;
    r.cnt = r.i1 < nc ? 2 : 1;
    r.w = 0.5f;
  }
  return r;
}

__device__ __forceinline__ float prolong_at(const Dims& c, const Dims& f, const float* __restrict__ src, int j) {
  const int jx = j % f.n[0], jy = (j / f.n[0]) % f.n[1], jz = j / (f.n[0] * f.n[1]);
  const Lin1 X = lin1(jx, c.n[0]), Y = lin1(jy, c.n[1]), Z = lin1(jz, c.n[2]);
  const float w = X.w * Y.w * Z.w;
  float acc = 0.f;
  for (int b = 0; b < Z.cnt; ++b)
    for (int a = 0; a < Y.cnt; ++a)
      for (int e = 0; e < X.cnt; ++e)
        acc = fmaf(w, __ldg(src + (e ? X.i1 : X.i0) + c.n[0] * ((a ? Y.i1 : Y.i0) + c.n[1] * (b ? Z.i1 : Z.i0))),
                   acc);
  return acc;
}

// fine[ch][j] (+)= scale * sum_i w'(j - 2i) coarse[ch][i] (P = 8 R^T, trilinear)
__global__ void k_prolong(int C, Dims c, Dims f, const float* __restrict__ coarse, float* __restrict__ fine,
                          float scale, int accumulate) {
  const int nc = (int)c.size(), nf = (int)f.size();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < C * nf; v += gridDim.x * blockDim.x) {
    const int ch = v / nf, j = v - ch * nf;
    const float val = scale * prolong_at(c, f, coarse + (size_t)ch * nc, j);
    if (accumulate) fine[(size_t)ch * nf + j] += val;
    else fine[(size_t)ch * nf + j] = val;
  }
}

// decoder step below the top level: out = (h + scale * P gx) * s, all kC channels; one
// thread per fine voxel (the neighbour indices are formed once for the 8 channels)
__global__ void k_prolong_gate(Dims c, Dims f, const float* __restrict__ gx, const float* __restrict__ h,
                               const float* __restrict__ s, float scale, float* __restrict__ out) {
  const int nc = (int)c.size(), nf = (int)f.size();
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nf; j += gridDim.x * blockDim.x) {
    const int jx = j % f.n[0], jy = (j / f.n[0]) % f.n[1], jz = j / (f.n[0] * f.n[1]);
    const Lin1 X = lin1(jx, c.n[0]), Y = lin1(jy, c.n[1]), Z = lin1(jz, c.n[2]);
    const float w = X.w * Y.w * Z.w;
    float acc[kC];
#pragma unroll
    for (int ch = 0; ch < kC; ++ch) acc[ch] = 0.f;
    for (int b = 0; b < Z.cnt; ++b)
      for (int a = 0; a < Y.cnt; ++a)
        for (int e = 0; e < X.cnt; ++e) {
          const int u = (e ? X.i1 : X.i0) + c.n[0] * ((a ? Y.i1 : Y.i0) + c.n[1] * (b ? Z.i1 : Z.i0));
#pragma unroll
          for (int ch = 0; ch < kC; ++ch) acc[ch] = fmaf(w, __ldg(gx + (size_t)ch * nc + u), acc[ch]);
        }
#pragma unroll
    for (int ch = 0; ch < kC; ++ch) {
      const size_t o = (size_t)ch * nf + j;
      out[o] = fmaf(scale, acc[ch], __ldg(h + o)) * __ldg(s + o);
    }
  }
}

// coarse-start input on the lattice: coarse[i] = sum_o w(o) dsq[2i+o] r[2i+o]
__global__ void k_scale_restrict(Dims f, Dims c, const float* __restrict__ r, const float* __restrict__ dsq,
                                 float* __restrict__ coarse) {
  const int nc = (int)c.size();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    const int ix = i % c.n[0], iy = (i / c.n[0]) % c.n[1], iz = i / (c.n[0] * c.n[1]);
    float acc = 0.f;
#pragma unroll
    for (int oz = -1; oz <= 1; ++oz) {
      const int fz = 2 * iz + oz;
      if (fz < 0 || fz >= f.n[2]) continue;
#pragma unroll
      for (int oy = -1; oy <= 1; ++oy) {
        const int fy = 2 * iy + oy;
        if (fy < 0 || fy >= f.n[1]) continue;
#pragma unroll
        for (int ox = -1; ox <= 1; ++ox) {
          const int fx = 2 * ix + ox;
          if (fx < 0 || fx >= f.n[0]) continue;
          const float w = (ox == 0 ? 0.5f : 0.25f) * (oy == 0 ? 0.5f : 0.25f) * (oz == 0 ? 0.5f : 0.25f);
          const int u = fx + f.n[0] * (fy + f.n[1] * fz);
          acc = fmaf(w, __ldg(dsq + u) * __ldg(r + u), acc);
        }
      }
    }
    coarse[i] = acc;
  }
}

// coarse-start output on the lattice: z[j] = dinv[j] r[j] + dsq[j] (P zc)[j] / 8
__global__ void k_prolong_out_lattice(Dims c, Dims f, const float* __restrict__ zc, const float* __restrict__ r,
                                      const float* __restrict__ dinv, const float* __restrict__ dsq,
                                      float* __restrict__ z) {
  const int nf = (int)f.size();
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nf; j += gridDim.x * blockDim.x)
    z[j] = fmaf(__ldg(dsq + j), 0.125f * prolong_at(c, f, zc, j), __ldg(dinv + j) * __ldg(r + j));
}

// ---- direct convolution for the coarse levels ------------------------------------------------
// SPLIT lanes per (voxel, output channel), CI / SPLIT input channels each: a lane runs
// the 27 taps of its channels and the SPLIT lanes add their sums with a shuffle tree.
// SPLIT = CI (one channel per lane) cuts the serial load chain of an output from
// CI x 27 to 27 and fills the GPU on the smallest levels; SPLIT = 1 keeps a warp on 32
// consecutive voxels of one channel plane (coalesced) for the larger coarse levels.
// Coarse lattices are too small to fill the GPU with tiles of 512 voxels, and a tiled
// CTA there runs long serial loops.  Outputs are channel-major; the weights are staged
// in shared memory per block.
template <int CI, int SPLIT, int LD, int EP>
__global__ void __launch_bounds__(kLT) k_conv_direct(TConvArgsS a) {
  static_assert(CI % SPLIT == 0 && (SPLIT & (SPLIT - 1)) == 0 && SPLIT <= 32, "lane split");
  constexpr int CPL = CI / SPLIT;   // input channels per lane
  __shared__ float sw[kC * CI * kTaps];   // [co][ci][tap] in the orientation applied
  for (int i = threadIdx.x; i < a.co_n * CI * kTaps; i += blockDim.x) {
    const int tap = i % kTaps, ci = (i / kTaps) % CI, co = i / (kTaps * CI);
    sw[i] = a.adjoint ? a.W[(ci * a.co_n + co) * kTaps + (kTaps - 1 - tap)] : a.W[(co * CI + ci) * kTaps + tap];
  }
  __syncthreads();
  const int nx = a.d.n[0], ny = a.d.n[1], nz = a.d.n[2];
  const int nv = nx * ny * nz;
  const int total = a.co_n * nv * SPLIT;   // a multiple of SPLIT; the stride is too, so a lane group is all in or all out
  const unsigned gmask = SPLIT >= 32 ? 0xffffffffu : (((1u << SPLIT) - 1u) << ((threadIdx.x & 31) & ~(SPLIT - 1)));
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int sub = idx % SPLIT, ov = idx / SPLIT;
    const int co = ov / nv, v = ov - co * nv;
    const int x = v % nx, y = (v / nx) % ny, z = v / (nx * ny);
    float acc = 0.f;
#pragma unroll
    for (int tap = 0; tap < kTaps; ++tap) {
      const int xx = x + tap % 3 - 1, yy = y + (tap / 3) % 3 - 1, zz = z + tap / 9 - 1;
      if ((unsigned)xx >= (unsigned)nx || (unsigned)yy >= (unsigned)ny || (unsigned)zz >= (unsigned)nz) continue;
      const int u = xx + nx * (yy + ny * zz);
#pragma unroll
      for (int cj = 0; cj < CPL; ++cj) {
        const int ci = sub * CPL + cj;
        float val = __ldg(a.in + (size_t)ci * nv + u);
        if (LD == LD_GATED) val *= __ldg(a.in_gate + (size_t)ci * nv + u);
        acc = fmaf(sw[(co * CI + ci) * kTaps + tap], val, acc);
      }
    }
#pragma unroll
    for (int o = SPLIT / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(gmask, acc, o, SPLIT);
    if (sub == 0) {
      if (EP == EP_GATE) acc *= __ldg(a.out_gate + (size_t)co * nv + v);
      a.out[(size_t)co * nv + v] = acc;
    }
  }
}

// ---- tiled convolution for the preconditioner application ---------------------------------
// Each CTA computes a TX x TY x TZ block of output voxels for all CO channels from a
// shared-memory copy of the (TX+2)(TY+2)(TZ+2) input halo (all CI channels) and of the
// weights laid out [ci][tap][co]; each thread holds XT consecutive x-voxels in registers so
// a weight fetched from shared memory feeds XT FMAs and an input row feeds 3 taps.
//   load modes : LD_PLAIN  in[ci][u]
//                LD_GATED  in[ci][u] * in_gate[ci][u]              (decoder, top level)
//                LD_GATHER sqrt(dinv[g]) r[g] at g = node_gid[u]    (encoder, level 0; CI = 1)
//   epilogues  : EP_GATE   out[co][v] = acc * out_gate[co][v]       (encoder)
//                EP_PLAIN  out[co][v] = acc                         (decoder)
//                EP_OUT    z[g] = dinv[g] r[g] + sqrt(dinv[g]) acc  (decoder, level 0; CO = 1)
//                EP_OUTLAT z[v] = dinv[v] r[v] + dsq[v] acc         (same, vectors on the lattice)

constexpr int kTX = 16, kTY = 8;

struct TConvArgs {
  Dims d;
  const float* in;
  const float* in_gate;
  const float* W;   // forward layout [co_f][ci_f][27]
  int adjoint;      // 1: apply the adjoint of the forward convolution W
  const float* out_gate;
  float* out;
  const int32_t* node_gid;
  const float* r;
  const float* dinv;
  const float* dsq;
  float* z;
};

// Halo rows are padded to a multiple of 4 floats (HXP) so a thread reads the XT + 2 = 6
// inputs of a row as one float4 and one float2; single-output-channel weights are stored
// [ci][dz][dy][4] (dx = 0..2, slot 3 zero) and read as one float4 per row.
template <int CI, int CO, int XT, int TZ>
struct TConvShape {
  static constexpr int HX = kTX + 2, HY = kTY + 2, HZ = TZ + 2;
  static constexpr int HXP = (HX + 3) & ~3;
  static constexpr int HP = HXP * HY * HZ;
  static constexpr int LX = kTX / XT;
  static constexpr int threads = LX * kTY * TZ;
  static constexpr int nw = CO == 1 ? CI * 9 * 4 : CI * kTaps * CO;
  static constexpr size_t smem = sizeof(float) * (size_t)(nw + CI * HP);
};

template <int CI, int CO, int XT, int TZ, int LD, int EP>
__global__ void __launch_bounds__(TConvShape<CI, CO, XT, TZ>::threads) k_tconv(TConvArgs a) {
  using S = TConvShape<CI, CO, XT, TZ>;
  extern __shared__ __align__(16) float tsm[];
  float* sw = tsm;          // [ci][tap][co]
  float* sx = tsm + S::nw;  // [ci][hz][hy][hx]
  const int nx = a.d.n[0], ny = a.d.n[1], nz = a.d.n[2];
  const int nv = nx * ny * nz;
  const int tiles_x = (nx + kTX - 1) / kTX, tiles_y = (ny + kTY - 1) / kTY;
  const int bx = blockIdx.x % tiles_x, by = (blockIdx.x / tiles_x) % tiles_y, bz = blockIdx.x / (tiles_x * tiles_y);
  const int x0 = bx * kTX, y0 = by * kTY, z0 = bz * TZ;
  for (int i = threadIdx.x; i < S::nw; i += S::threads) {
    int co, tap, ci;
    if (CO == 1) {   // [ci][dz][dy][4]
      const int dx = i % 4, row = (i / 4) % 9;
      ci = i / 36;
      co = 0;
      tap = dx < 3 ? row * 3 + dx : -1;
    } else {
      co = i % CO;
      tap = (i / CO) % kTaps;
      ci = i / (kTaps * CO);
    }
    sw[i] = tap < 0 ? 0.f
                    : (a.adjoint ? a.W[(ci * CO + co) * kTaps + (kTaps - 1 - tap)] : a.W[(co * CI + ci) * kTaps + tap]);
  }
  // halo: U elements per thread per step, all loads issued before any is used, so a CTA
  // waits for a few load latencies instead of one per element (the gathered level-0 input
  // is a node -> gid -> value chain)
  constexpr int U = CI == 1 ? 8 : 2;
  for (int i0 = threadIdx.x; i0 < S::HP; i0 += S::threads * U) {
    int uu[U];
    bool inb[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int i = i0 + k * S::threads;
      const int hx = i % S::HXP, hy = (i / S::HXP) % S::HY, hz = i / (S::HXP * S::HY);
      const int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = z0 + hz - 1;
      inb[k] = i < S::HP && hx < S::HX && gx >= 0 && gx < nx && gy >= 0 && gy < ny && gz >= 0 && gz < nz;
      uu[k] = inb[k] ? gx + nx * (gy + ny * gz) : 0;
    }
    if (LD == LD_GATHER) {
      int32_t gg[U];
#pragma unroll
      for (int k = 0; k < U; ++k) gg[k] = inb[k] ? __ldg(a.node_gid + uu[k]) : -1;
      float dv[U], rv[U];
#pragma unroll
      for (int k = 0; k < U; ++k) {
        dv[k] = gg[k] >= 0 ? __ldg(a.dinv + gg[k]) : 0.f;
        rv[k] = gg[k] >= 0 ? __ldg(a.r + gg[k]) : 0.f;
      }
#pragma unroll
      for (int k = 0; k < U; ++k) {
        const int i = i0 + k * S::threads;
        if (i < S::HP) sx[i] = gg[k] >= 0 ? sqrtf(dv[k]) * rv[k] : 0.f;
      }
    } else {
      float v[U][CI];
#pragma unroll
      for (int k = 0; k < U; ++k)
#pragma unroll
        for (int ci = 0; ci < CI; ++ci) {
          v[k][ci] = inb[k] ? __ldg(a.in + (size_t)ci * nv + uu[k]) : 0.f;
          if (LD == LD_GATED && inb[k]) v[k][ci] *= __ldg(a.in_gate + (size_t)ci * nv + uu[k]);
        }
#pragma unroll
      for (int k = 0; k < U; ++k) {
        const int i = i0 + k * S::threads;
        if (i < S::HP)
#pragma unroll
          for (int ci = 0; ci < CI; ++ci) sx[ci * S::HP + i] = v[k][ci];
      }
    }
  }
  __syncthreads();
  const int tx = threadIdx.x % S::LX, ty = (threadIdx.x / S::LX) % kTY, tz = threadIdx.x / (S::LX * kTY);
  float acc[XT][CO];
#pragma unroll
  for (int j = 0; j < XT; ++j)
#pragma unroll
    for (int co = 0; co < CO; ++co) acc[j][co] = 0.f;
#pragma unroll 1
  for (int ci = 0; ci < CI; ++ci) {
#pragma unroll
    for (int dz = 0; dz < 3; ++dz)
#pragma unroll
      for (int dy = 0; dy < 3; ++dy) {
        const float* row = sx + ci * S::HP + (tz + dz) * (S::HXP * S::HY) + (ty + dy) * S::HXP + tx * XT;
        float v[XT + 2];
        if constexpr (XT == 4) {
          const float4 a4 = *reinterpret_cast<const float4*>(row);
          const float2 b2 = *reinterpret_cast<const float2*>(row + 4);
          v[0] = a4.x;
          v[1] = a4.y;
          v[2] = a4.z;
          v[3] = a4.w;
          v[4] = b2.x;
          v[5] = b2.y;
        } else {
#pragma unroll
          for (int k = 0; k < XT + 2; ++k) v[k] = row[k];
        }
        float w1[4];
        if constexpr (CO == 1) {
          const float4 t = *reinterpret_cast<const float4*>(sw + (ci * 9 + dz * 3 + dy) * 4);
          w1[0] = t.x;
          w1[1] = t.y;
          w1[2] = t.z;
          w1[3] = t.w;
        }
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
          const float* wp = sw + (ci * kTaps + dz * 9 + dy * 3 + dx) * CO;
          float w[CO];
          if constexpr (CO == 1) {
            w[0] = w1[dx];
          } else if constexpr (CO % 4 == 0) {
#pragma unroll
            for (int q = 0; q < CO / 4; ++q) {
              const float4 t = reinterpret_cast<const float4*>(wp)[q];
              w[4 * q] = t.x;
              w[4 * q + 1] = t.y;
              w[4 * q + 2] = t.z;
              w[4 * q + 3] = t.w;
            }
          } else {
#pragma unroll
            for (int co = 0; co < CO; ++co) w[co] = wp[co];
          }
#pragma unroll
          for (int j = 0; j < XT; ++j)
#pragma unroll
            for (int co = 0; co < CO; ++co) acc[j][co] = fmaf(w[co], v[j + dx], acc[j][co]);
        }
      }
  }
  const int y = y0 + ty, zz = z0 + tz;
  if (y >= ny || zz >= nz) return;
#pragma unroll
  for (int j = 0; j < XT; ++j) {
    const int x = x0 + tx * XT + j;
    if (x >= nx) break;
    const int v = x + nx * (y + ny * zz);
    if (EP == EP_OUTLAT) {
      a.z[v] = fmaf(__ldg(a.dsq + v), acc[j][0], __ldg(a.dinv + v) * __ldg(a.r + v));
    } else if (EP == EP_OUT) {
      const int32_t g = __ldg(a.node_gid + v);
      if (g >= 0) {
        const float di = __ldg(a.dinv + g);
        a.z[g] = fmaf(sqrtf(di), acc[j][0], di * __ldg(a.r + g));
      }
    } else {
#pragma unroll
      for (int co = 0; co < CO; ++co) {
        float o = acc[j][co];
        if (EP == EP_GATE) o *= __ldg(a.out_gate + (size_t)co * nv + v);
        a.out[(size_t)co * nv + v] = o;
      }
    }
  }
}

// ---- elementwise ---------------------------------------------------------------------------
__global__ void k_sigmoid(int64_t n, float* __restrict__ a) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = 1.f / (1.f + __expf(-a[i]));
}
// gy -> grad of the pre-gate value (ga = gy*s) and of the gate pre-activation (gp = gy*a*s*(1-s));
// a = ungated value.
__global__ void k_gate_bwd(int64_t n, const float* __restrict__ gy, const float* __restrict__ a,
                           const float* __restrict__ s, float* __restrict__ ga, float* __restrict__ gp) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float si = s[i];
    ga[i] = gy[i] * si;
    if (gp) gp[i] = gy[i] * a[i] * si * (1.f - si);
  }
}
__global__ void k_mul(int64_t n, const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ c) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c[i] = a[i] * b[i];
}
__global__ void k_copyf(int64_t n, const float* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

// lattice[X] = scale * dinv[gid] * v[gid] (0 on Dirichlet nodes); v in gid order
__global__ void k_to_lattice(int64_t nlat, const int32_t* __restrict__ node_gid, const float* __restrict__ v,
                             const float* __restrict__ dinv, float* __restrict__ lat) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nlat; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t g = node_gid[i];
    lat[i] = g >= 0 ? (dinv ? dinv[g] * v[g] : v[g]) : 0.f;
  }
}
// out[r] = a[X_r] + b[X_r] over the owned rows (X_r = row_node[r]); b may be null
__global__ void k_from_lattice(int64_t n, const int32_t* __restrict__ row_node, const float* __restrict__ a,
                               const float* __restrict__ b, float* __restrict__ out) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t X = row_node[r];
    out[r] = a[X] + (b ? b[X] : 0.f);
  }
}

// node feature: log of the mean coefficient of the valid cells around the node (cube Q1:
// w = K2 * kappa, so kappa = w / K2)
__global__ void k_node_logk(Dims d, const int64_t* __restrict__ ncell, const double* __restrict__ w, double inv_k2,
                            float* __restrict__ f) {
  const int64_t nv = d.size();
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(v % d.n[0]), y = (int)((v / d.n[0]) % d.n[1]), z = (int)(v / ((int64_t)d.n[0] * d.n[1]));
    double s = 0.0;
    int c = 0;
    for (int a = 0; a < 8; ++a) {
      const int64_t cx = x - 1 + (a & 1), cy = y - 1 + ((a >> 1) & 1), cz = z - 1 + ((a >> 2) & 1);
      if (cx < 0 || cx >= ncell[0] || cy < 0 || cy >= ncell[1] || cz < 0 || cz >= ncell[2]) continue;
      s += w[cx + ncell[0] * (cy + ncell[1] * cz)] * inv_k2;
      ++c;
    }
    f[v] = c ? (float)log(s / c) : 0.f;
  }
}

// Adam on the flat parameter vector
__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2, float scale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] * scale;
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// y = s * (a - b) (gid order)
__global__ void k_axmb(int64_t n, float s, const float* __restrict__ a, const float* __restrict__ b,
                       float* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = s * (a[i] - (b ? b[i] : 0.f));
}

__device__ inline double blk_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  return s;
}
__global__ void k_sum_d(int nb, const double* __restrict__ p, double* __restrict__ out) {
  __shared__ double sh[kLT / 32];
  double a = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) a += p[i];
  const double s = blk_sum(a, sh);
  if (threadIdx.x == 0) *out = s;
}

static inline unsigned nb_for(int64_t n) {
  int64_t b = (n + kLT - 1) / kLT;
  return (unsigned)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}


// lattice[X] = sc[X] * v[gid(X)] (0 on Dirichlet nodes); v in gid order
__global__ void k_to_lattice_scaled(int64_t nlat, const int32_t* __restrict__ node_gid, const float* __restrict__ v,
                                    const float* __restrict__ sc, float* __restrict__ lat) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nlat; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t g = node_gid[i];
    lat[i] = g >= 0 ? sc[i] * v[g] : 0.f;
  }
}
// dsq[X] = sqrt(dinv[gid(X)]) at free nodes, 0 elsewhere
__global__ void k_dsqrt_lattice(int64_t nlat, const int32_t* __restrict__ node_gid, const float* __restrict__ dinv,
                                float* __restrict__ dsq) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nlat; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t g = node_gid[i];
    dsq[i] = g >= 0 ? sqrtf(dinv[g]) : 0.f;
  }
}
// z[r] = dinv[r] v[r] + dsq[X_r] zl[X_r] over the owned rows
__global__ void k_learned_out(int64_t n, const int32_t* __restrict__ row_node, const float* __restrict__ dinv,
                              const float* __restrict__ v, const float* __restrict__ dsq, const float* __restrict__ zl,
                              float* __restrict__ z) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t X = row_node[r];
    z[r] = dinv[r] * v[r] + dsq[X] * zl[X];
  }
}

}  // namespace gd

using namespace gd;

constexpr int kMaxLevels = 6;

// ---------------------------------------------------------------------------------
// Network object
// ---------------------------------------------------------------------------------
struct gd_learned {
  gd_asm* A = nullptr;
  int levels = 3;
  Dims L[kMaxLevels];
  int64_t nl[kMaxLevels] = {0};
  int64_t nparams = 0;
  int offW[kMaxLevels] = {0}, offG[kMaxLevels] = {0}, offB[kMaxLevels] = {0};
  DBuf<float> params, grads, adam_m, adam_v;
  int64_t adam_t = 0;
  DBuf<float> f[kMaxLevels], s[kMaxLevels];   // features (1 ch) and gates (8 ch)
  DBuf<float> dsq;                            // lattice sqrt(D^-1) (0 on Dirichlet nodes)
  // encoder caches of the two inputs used in training (path 0: D^-1/2 r, path 1: the
  // loss gradient); the decoder and the backward pass use the scratch maps below
  DBuf<float> x[2][kMaxLevels], a[2][kMaxLevels], h[2][kMaxLevels];
  DBuf<float> u[kMaxLevels], gx[kMaxLevels], d[kMaxLevels], da[kMaxLevels], gp[kMaxLevels];
  DBuf<float> zl;
  // coarse start: the network's level 0 is the once-restricted lattice
  int cs = 0;
  Dims LF{};          // node lattice
  int64_t nlf = 0;
  DBuf<float> xf, zf;   // node-lattice scratch (restriction input, prolongation output)
  DBuf<float> part;
  DBuf<double> dred;
  DBuf<float> zv, ev, dv, yv;
  bool prepared = false;
  int64_t prepared_epoch = -1;
  uint64_t serial = 0;   // unique per object (key of the solver's captured graphs)
};

namespace gd {

static int conv_launch(int ci, int co, const Dims& d, const float* in, const float* W, const float* gate,
                       const float* bias, float* out, int mode, int acc, cudaStream_t st) {
  const unsigned nb = nb_for(d.size());
  if (ci == 1 && co == 8) k_conv3<1, 8><<<nb, kLT, 0, st>>>(d, in, W, gate, bias, out, mode, acc);
  else if (ci == 8 && co == 8) k_conv3<8, 8><<<nb, kLT, 0, st>>>(d, in, W, gate, bias, out, mode, acc);
  else if (ci == 8 && co == 1) k_conv3<8, 1><<<nb, kLT, 0, st>>>(d, in, W, gate, bias, out, mode, acc);
  else return fail(GD_ERR_UNSUPPORTED, "learned: unsupported convolution shape");
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

static int ntiles(const Dims& d) {
  return ((d.n[0] + kTile - 1) / kTile) * ((d.n[1] + kTile - 1) / kTile) * ((d.n[2] + kTile - 1) / kTile);
}

// dW += wgrad(in, g); W has shape [co][ci][27]
static int wgrad_launch(gd_learned* N, int ci, int co, const Dims& d, const float* in, const float* g, float* dW,
                        cudaStream_t st) {
  const int nt = ntiles(d);
  const int nw = ci * co * kTaps;
  if (N->part.n < (size_t)nt * nw) GD_TRY(dalloc(N->part, (size_t)nt * nw));
  if (ci == 1 && co == 8) k_conv3_wgrad<1, 8><<<nt, kLT, 0, st>>>(d, in, g, N->part.p);
  else if (ci == 8 && co == 8) k_conv3_wgrad<8, 8><<<nt, kLT, 0, st>>>(d, in, g, N->part.p);
  else return fail(GD_ERR_UNSUPPORTED, "learned: unsupported gradient shape");
  k_sum_partials<<<(nw + 127) / 128, 128, 0, st>>>(nt, nw, N->part.p, dW);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

static int bgrad_launch(gd_learned* N, const Dims& d, const float* g, float* dB, cudaStream_t st) {
  const int nb = 256;
  if (N->part.n < (size_t)nb * kC) GD_TRY(dalloc(N->part, (size_t)nb * kC));
  k_bias_grad<<<nb, kLT, 0, st>>>(d, kC, g, N->part.p);
  k_sum_partials<<<1, 128, 0, st>>>(nb, kC, N->part.p, dB);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

static inline int cin_of(int l) { return l == 0 ? 1 : kC; }

// static part: features, gates and the diagonal scaling (after every numeric assembly)
static int net_prepare(gd_learned* N, cudaStream_t st) {
  gd_asm* A = N->A;
  if (N->prepared && N->prepared_epoch == A->numeric_epoch) return GD_OK;
  GD_TRY(mixed_setup(A));
  const Geom& g = A->test->geom;
  int64_t hn[3] = {g.n[0], g.n[1], g.n[2]};
  DBuf<int64_t> dn;
  GD_TRY(dalloc(dn, 3));
  GD_CUDA_TRY(cudaMemcpyAsync(dn.p, hn, sizeof(hn), cudaMemcpyHostToDevice, st));
  const float* P = N->params.p;
  const float* dinv = A->mx.f32.p + 5 * A->ngdofs;
  if (N->cs) {
    k_node_logk<<<nb_for(N->nlf), kLT, 0, st>>>(N->LF, dn.p, A->w_cells.p, 1.0 / A->mf_k2, N->xf.p);
    k_restrict<<<nb_for(N->nl[0]), kLT, 0, st>>>(1, N->LF, N->L[0], N->xf.p, N->f[0].p, 1.f);
  } else {
    k_node_logk<<<nb_for(N->nl[0]), kLT, 0, st>>>(N->L[0], dn.p, A->w_cells.p, 1.0 / A->mf_k2, N->f[0].p);
  }
  for (int l = 1; l < N->levels; ++l)
    k_restrict<<<nb_for(N->nl[l]), kLT, 0, st>>>(1, N->L[l - 1], N->L[l], N->f[l - 1].p, N->f[l].p, 1.f);
  GD_CUDA_TRY(cudaGetLastError());
  for (int l = 0; l < N->levels; ++l) {
    GD_TRY(conv_launch(1, 8, N->L[l], N->f[l].p, P + N->offG[l], nullptr, P + N->offB[l], N->s[l].p, 0, 0, st));
    k_sigmoid<<<nb_for(kC * N->nl[l]), kLT, 0, st>>>(kC * N->nl[l], N->s[l].p);
  }
  k_dsqrt_lattice<<<nb_for(N->nlf), kLT, 0, st>>>(N->nlf, A->mx.node_gid.p, dinv, N->dsq.p);
  GD_CUDA_TRY(cudaGetLastError());
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  dfreeb(dn);
  N->prepared = true;
  N->prepared_epoch = A->numeric_epoch;
  return GD_OK;
}

// encoder of path p on the lattice input x[p][0]: h[p][l] = conv(x_l; W_l) * s_l
static int net_encode(gd_learned* N, int p, cudaStream_t st) {
  const float* P = N->params.p;
  for (int l = 0; l < N->levels; ++l) {
    if (l > 0)
      k_restrict<<<nb_for(kC * N->nl[l]), kLT, 0, st>>>(kC, N->L[l - 1], N->L[l], N->h[p][l - 1].p, N->x[p][l].p,
                                                        1.f);
    GD_TRY(conv_launch(cin_of(l), kC, N->L[l], N->x[p][l].p, P + N->offW[l], nullptr, nullptr, N->a[p][l].p, 0, 0, st));
    k_mul<<<nb_for(kC * N->nl[l]), kLT, 0, st>>>(kC * N->nl[l], N->a[p][l].p, N->s[l].p, N->h[p][l].p);
  }
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

// decoder: zl = S^T (h[p][0..L-1])  (the adjoint of the encoder, summed over levels)
static int net_decode(gd_learned* N, int p, cudaStream_t st) {
  const float* P = N->params.p;
  const int Lv = N->levels;
  k_copyf<<<nb_for(kC * N->nl[Lv - 1]), kLT, 0, st>>>(kC * N->nl[Lv - 1], N->h[p][Lv - 1].p, N->u[Lv - 1].p);
  for (int l = Lv - 1; l >= 0; --l) {
    k_mul<<<nb_for(kC * N->nl[l]), kLT, 0, st>>>(kC * N->nl[l], N->u[l].p, N->s[l].p, N->da[l].p);
    float* out = l == 0 ? N->zl.p : N->gx[l].p;
    GD_TRY(conv_launch(kC, cin_of(l), N->L[l], N->da[l].p, P + N->offW[l], nullptr, nullptr, out, 1, 0, st));
    if (l > 0) {
      k_copyf<<<nb_for(kC * N->nl[l - 1]), kLT, 0, st>>>(kC * N->nl[l - 1], N->h[p][l - 1].p, N->u[l - 1].p);
      k_prolong<<<nb_for(kC * N->nl[l - 1]), kLT, 0, st>>>(kC, N->L[l], N->L[l - 1], N->gx[l].p, N->u[l - 1].p,
                                                           0.125f, 1);
    }
  }
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

// backward of the encoder of path p with cotangents (h[q][l]) at every level; accumulates
// W, G, b gradients
static int net_encoder_backward(gd_learned* N, int p, int q, cudaStream_t st) {
  const float* P = N->params.p;
  float* G = N->grads.p;
  const int Lv = N->levels;
  k_copyf<<<nb_for(kC * N->nl[Lv - 1]), kLT, 0, st>>>(kC * N->nl[Lv - 1], N->h[q][Lv - 1].p, N->d[Lv - 1].p);
  for (int l = Lv - 1; l >= 0; --l) {
    const int64_t m = kC * N->nl[l];
    k_gate_bwd<<<nb_for(m), kLT, 0, st>>>(m, N->d[l].p, N->a[p][l].p, N->s[l].p, N->da[l].p, N->gp[l].p);
    GD_TRY(wgrad_launch(N, 1, kC, N->L[l], N->f[l].p, N->gp[l].p, G + N->offG[l], st));
    GD_TRY(bgrad_launch(N, N->L[l], N->gp[l].p, G + N->offB[l], st));
    GD_TRY(wgrad_launch(N, cin_of(l), kC, N->L[l], N->x[p][l].p, N->da[l].p, G + N->offW[l], st));
    if (l > 0) {
      GD_TRY(conv_launch(kC, kC, N->L[l], N->da[l].p, P + N->offW[l], nullptr, nullptr, N->gx[l].p, 1, 0, st));
      k_copyf<<<nb_for(kC * N->nl[l - 1]), kLT, 0, st>>>(kC * N->nl[l - 1], N->h[q][l - 1].p, N->d[l - 1].p);
      k_prolong<<<nb_for(kC * N->nl[l - 1]), kLT, 0, st>>>(kC, N->L[l], N->L[l - 1], N->gx[l].p, N->d[l - 1].p,
                                                           0.125f, 1);
    }
  }
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

// z = D^-1 r + D^-1/2 S^T S D^-1/2 r  (r, z in gid order); keeps the path-0 encoder cache
// network input of path p from a gid-order vector v: x_0 = (R) D^-1/2 v
static int net_input(gd_learned* N, int p, const float* v, cudaStream_t st) {
  gd_asm* A = N->A;
  float* fine = N->cs ? N->xf.p : N->x[p][0].p;
  k_to_lattice_scaled<<<nb_for(N->nlf), kLT, 0, st>>>(N->nlf, A->mx.node_gid.p, v, N->dsq.p, fine);
  if (N->cs) k_restrict<<<nb_for(N->nl[0]), kLT, 0, st>>>(1, N->LF, N->L[0], N->xf.p, N->x[p][0].p, 1.f);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

static int net_forward(gd_learned* N, const float* r, float* z, cudaStream_t st) {
  gd_asm* A = N->A;
  const float* dinv = A->mx.f32.p + 5 * A->ngdofs;
  GD_TRY(net_input(N, 0, r, st));
  GD_TRY(net_encode(N, 0, st));
  GD_TRY(net_decode(N, 0, st));
  const float* zo = N->zl.p;
  if (N->cs) {   // R^T = P / 8
    k_prolong<<<nb_for(N->nlf), kLT, 0, st>>>(1, N->L[0], N->LF, N->zl.p, N->zf.p, 0.125f, 0);
    zo = N->zf.p;
  }
  k_learned_out<<<nb_for(A->ngdofs), kLT, 0, st>>>(A->ngdofs, A->row_node.p, dinv, r, N->dsq.p, zo, z);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

// parameter gradient of <gz, z(r)> (gz = dL/dz in gid order), accumulated into grads
static int net_backward(gd_learned* N, const float* gz, cudaStream_t st) {
  gd_asm* A = N->A;
  // path 1 input: (R) D^-1/2 gz
  (void)A;
  GD_TRY(net_input(N, 1, gz, st));
  GD_TRY(net_encode(N, 1, st));
  // d<g, S^T S x> = <S g, dS x> + <S x, dS g>
  GD_TRY(net_encoder_backward(N, 0, 1, st));
  GD_TRY(net_encoder_backward(N, 1, 0, st));
  return GD_OK;
}

// loss for one pair and its gradient wrt z: L = (z-e)A(z-e) / eAe, gz = 2 A(z-e) / eAe
static int net_loss(gd_learned* N, const float* z, const float* e, double* loss, float* gz, cudaStream_t st) {
  gd_asm* A = N->A;
  const int64_t n = A->ngdofs;
  double* red = N->dred.p;   // [0..1023] partials, [2048] eAe, [2049] dAd
  k_axmb<<<nb_for(n), kLT, 0, st>>>(n, 1.f, z, e, N->dv.p);
  GD_TRY(mixed_apply(A, N->dv.p, N->yv.p, red, st));   // yv = A d, partial d.Ad
  const int nbm = (int)std::min<int64_t>((n + 255) / 256, 1024);
  k_sum_d<<<1, kLT, 0, st>>>(nbm, red, red + 2049);
  GD_TRY(mixed_apply(A, e, N->zv.p, red, st));         // partial e.Ae
  k_sum_d<<<1, kLT, 0, st>>>(nbm, red, red + 2048);
  double h[2];
  GD_CUDA_TRY(cudaMemcpyAsync(h, red + 2048, sizeof(h), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  const double eAe = h[0] > 0 ? h[0] : 1.0;
  *loss = h[1] / eAe;
  if (gz) {
    k_axmb<<<nb_for(n), kLT, 0, st>>>(n, (float)(2.0 / eAe), N->yv.p, nullptr, gz);
    GD_CUDA_TRY(cudaGetLastError());
  }
  return GD_OK;
}

// levels with fewer voxels than this use the direct convolution (one thread per voxel and
// output channel) instead of the shared-memory tiles
constexpr int64_t kDirectConvVoxels = 10000;
// levels below this (but above the direct limit) use 2 voxels per thread: twice the
// threads per tile, so a level of ~10^5 voxels still fills the SMs
constexpr int64_t kWideTileVoxels = 400000;

// levels with fewer voxels than this split the input channels of an output across lanes
constexpr int64_t kSplitConvVoxels = 8192;

template <int CI, int LD, int EP>
static int direct_launch(const Dims& d, const float* in, const float* in_gate, const float* W, int adjoint, int co_n,
                         const float* out_gate, float* out, cudaStream_t st) {
  TConvArgsS a{d, in, in_gate, W, adjoint, co_n, out_gate, out};
  if (d.size() < kSplitConvVoxels)
    k_conv_direct<CI, CI, LD, EP><<<nb_for((int64_t)co_n * d.size() * CI), kLT, 0, st>>>(a);
  else
    k_conv_direct<CI, 1, LD, EP><<<nb_for((int64_t)co_n * d.size()), kLT, 0, st>>>(a);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

template <int CI, int CO, int XT, int TZ, int LD, int EP>
static int tconv_launch(const TConvArgs& a, cudaStream_t st) {
  using S = TConvShape<CI, CO, XT, TZ>;
  auto kern = k_tconv<CI, CO, XT, TZ, LD, EP>;
  if (S::smem > 48 * 1024)
    GD_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::smem));
  const unsigned nb = (unsigned)(((a.d.n[0] + kTX - 1) / kTX) * ((a.d.n[1] + kTY - 1) / kTY) * ((a.d.n[2] + TZ - 1) / TZ));
  kern<<<nb, S::threads, S::smem, st>>>(a);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

// encoder convolution of level l with gates: out = conv(in; W_l) * s_l (CI input channels,
// 8 outputs); direct for coarse levels, tiles otherwise
template <int CI>
static int enc_conv(gd_learned* N, int l, const float* in, cudaStream_t st) {
  TConvArgs t{};
  t.d = N->L[l];
  t.in = in;
  t.W = N->params.p + N->offW[l];
  t.adjoint = 0;
  t.out_gate = N->s[l].p;
  t.out = N->h[0][l].p;
  if (N->nl[l] < kDirectConvVoxels)
    return direct_launch<CI, LD_PLAIN, EP_GATE>(t.d, in, nullptr, t.W, 0, kC, t.out_gate, t.out, st);
  if (CI == kC && N->nl[l] < kWideTileVoxels) return tconv_launch<CI, kC, 2, 4, LD_PLAIN, EP_GATE>(t, st);
  return tconv_launch<CI, kC, 4, 4, LD_PLAIN, EP_GATE>(t, st);
}

// decoder (adjoint) convolution of level l into CO outputs: in (8 channels, times the gates
// when LD == LD_GATED)
template <int CO, int LD>
static int dec_conv(gd_learned* N, int l, const float* in, const float* in_gate, float* out, cudaStream_t st) {
  TConvArgs t{};
  t.d = N->L[l];
  t.in = in;
  t.in_gate = in_gate;
  t.W = N->params.p + N->offW[l];
  t.adjoint = 1;
  t.out = out;
  if (N->nl[l] < kDirectConvVoxels)
    return direct_launch<kC, LD, EP_PLAIN>(t.d, in, in_gate, t.W, 1, CO, nullptr, out, st);
  if (CO == kC && N->nl[l] < kWideTileVoxels) return tconv_launch<kC, CO, 2, 4, LD, EP_PLAIN>(t, st);
  return tconv_launch<kC, CO, 4, 4, LD, EP_PLAIN>(t, st);
}

// z = D^-1 r + D^-1/2 (R^T) S^T S (R) D^-1/2 r for the solver (no training caches).
// `lattice`: r and z on the node lattice (0 on Dirichlet nodes), else in gid order.  On
// the full lattice the gather/scale of r and the output are fused into the level-0
// convolutions; with the coarse start they are fused into the restriction and the
// final prolongation instead.
static int net_apply(gd_learned* N, const float* r, float* z, bool lattice, cudaStream_t st) {
  gd_asm* A = N->A;
  const float* P = N->params.p;
  const int Lv = N->levels;
  const float* dinv = lattice ? lattice_dinv(A) : A->mx.f32.p + 5 * A->ngdofs;
  // encoder
  for (int l = 0; l < Lv; ++l) {
    if (l > 0) {
      k_restrict<<<nb_for(kC * N->nl[l]), kLT, 0, st>>>(kC, N->L[l - 1], N->L[l], N->h[0][l - 1].p, N->x[0][l].p, 1.f);
      GD_TRY((enc_conv<kC>(N, l, N->x[0][l].p, st)));
    } else if (N->cs) {
      if (lattice) {
        k_scale_restrict<<<nb_for(N->nl[0]), kLT, 0, st>>>(N->LF, N->L[0], r, N->dsq.p, N->x[0][0].p);
      } else {
        k_to_lattice_scaled<<<nb_for(N->nlf), kLT, 0, st>>>(N->nlf, A->mx.node_gid.p, r, N->dsq.p, N->xf.p);
        k_restrict<<<nb_for(N->nl[0]), kLT, 0, st>>>(1, N->LF, N->L[0], N->xf.p, N->x[0][0].p, 1.f);
      }
      GD_CUDA_TRY(cudaGetLastError());
      GD_TRY((enc_conv<1>(N, 0, N->x[0][0].p, st)));
    } else {
      TConvArgs t{};
      t.d = N->L[0];
      t.W = P + N->offW[0];
      t.out_gate = N->s[0].p;
      t.out = N->h[0][0].p;
      t.r = r;
      t.dinv = dinv;
      t.node_gid = A->mx.node_gid.p;
      if (lattice) {
        t.in = r;
        t.in_gate = N->dsq.p;
        GD_TRY((tconv_launch<1, kC, 4, 4, LD_GATED, EP_GATE>(t, st)));
      } else {
        GD_TRY((tconv_launch<1, kC, 4, 4, LD_GATHER, EP_GATE>(t, st)));
      }
    }
  }
  // decoder (adjoint convolutions)
  for (int l = Lv - 1; l >= 0; --l) {
    const bool top = l == Lv - 1;
    const float* in = top ? N->h[0][l].p : N->da[l].p;
    const float* gate = top ? N->s[l].p : nullptr;
    if (!top) {
      k_prolong_gate<<<nb_for(N->nl[l]), kLT, 0, st>>>(N->L[l + 1], N->L[l], N->gx[l + 1].p, N->h[0][l].p,
                                                       N->s[l].p, 0.125f, N->da[l].p);
      GD_CUDA_TRY(cudaGetLastError());
    }
    if (l > 0) {
      if (top) GD_TRY((dec_conv<kC, LD_GATED>(N, l, in, gate, N->gx[l].p, st)));
      else GD_TRY((dec_conv<kC, LD_PLAIN>(N, l, in, gate, N->gx[l].p, st)));
    } else if (N->cs) {
      if (top) GD_TRY((dec_conv<1, LD_GATED>(N, 0, in, gate, N->zl.p, st)));
      else GD_TRY((dec_conv<1, LD_PLAIN>(N, 0, in, gate, N->zl.p, st)));
      if (lattice) {
        k_prolong_out_lattice<<<nb_for(N->nlf), kLT, 0, st>>>(N->L[0], N->LF, N->zl.p, r, dinv, N->dsq.p, z);
      } else {
        k_prolong<<<nb_for(N->nlf), kLT, 0, st>>>(1, N->L[0], N->LF, N->zl.p, N->zf.p, 0.125f, 0);
        k_learned_out<<<nb_for(A->ngdofs), kLT, 0, st>>>(A->ngdofs, A->row_node.p, dinv, r, N->dsq.p, N->zf.p, z);
      }
      GD_CUDA_TRY(cudaGetLastError());
    } else {
      TConvArgs t{};
      t.d = N->L[0];
      t.in = in;
      t.in_gate = gate;
      t.W = P + N->offW[0];
      t.adjoint = 1;
      t.r = r;
      t.dinv = dinv;
      t.dsq = N->dsq.p;
      t.node_gid = A->mx.node_gid.p;
      t.z = z;
      if (lattice) {
        if (top) GD_TRY((tconv_launch<kC, 1, 4, 4, LD_GATED, EP_OUTLAT>(t, st)));
        else GD_TRY((tconv_launch<kC, 1, 4, 4, LD_PLAIN, EP_OUTLAT>(t, st)));
      } else {
        if (top) GD_TRY((tconv_launch<kC, 1, 4, 4, LD_GATED, EP_OUT>(t, st)));
        else GD_TRY((tconv_launch<kC, 1, 4, 4, LD_PLAIN, EP_OUT>(t, st)));
      }
    }
  }
  return GD_OK;
}

static int net_apply_fast(gd_learned* N, const float* r, float* z, cudaStream_t st) {
  return net_apply(N, r, z, false, st);
}

static int net_apply_lattice(gd_learned* N, const float* r, float* z, cudaStream_t st) {
  return net_apply(N, r, z, true, st);
}

static int apply_as_precond(void* ctx, gd_asm* A, const float* r, float* z, cudaStream_t st) {
  (void)A;
  return net_apply_fast(static_cast<gd_learned*>(ctx), r, z, st);
}

static int apply_as_precond_lattice(void* ctx, gd_asm* A, const float* r, float* z, cudaStream_t st) {
  (void)A;
  return net_apply_lattice(static_cast<gd_learned*>(ctx), r, z, st);
}

}  // namespace gd

// ---------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------
extern "C" int gd_learned_create(gd_asm* A, int levels, int flags, uint64_t seed, gd_learned** out) {
  if (!A || !out) return fail(GD_ERR_ARG, "gd_learned_create: null argument");
  if (levels < 1 || levels > kMaxLevels) return fail(GD_ERR_ARG, "gd_learned_create: levels must be 1..6");
  if (flags & ~GD_LEARNED_COARSE_START) return fail(GD_ERR_ARG, "gd_learned_create: unknown flags");
  if (!A->numeric_done) return fail(GD_ERR_STATE, "gd_learned_create: assemble the system first");
  if (!(A->fast_q1 && A->q1c_cube && A->test->geom.dim == 3) || A->qp_values)
    return fail(GD_ERR_UNSUPPORTED,
                "gd_learned_create: the learned preconditioner needs 3D Q1 on cube cells with cell-wise coefficients");
  const Geom& g = A->test->geom;
  if ((double)g.N[0] * g.N[1] * g.N[2] * kC >= 2147483647.0)
    return fail(GD_ERR_UNSUPPORTED, "gd_learned_create: node lattice too large (8 channels must index in 32 bits)");
  static std::atomic<uint64_t> next_serial{1};
  gd_learned* N = new gd_learned();
  N->serial = next_serial.fetch_add(1);
  N->A = A;
  N->levels = levels;
  N->cs = (flags & GD_LEARNED_COARSE_START) ? 1 : 0;
  for (int d = 0; d < 3; ++d) N->LF.n[d] = (int)g.N[d];
  N->nlf = N->LF.size();
  N->L[0] = N->cs ? coarse_dims(N->LF) : N->LF;
  for (int l = 1; l < levels; ++l) N->L[l] = coarse_dims(N->L[l - 1]);
  for (int l = 0; l < levels; ++l) N->nl[l] = N->L[l].size();
  int off = 0;
  for (int l = 0; l < levels; ++l) {
    N->offW[l] = off;
    off += kC * cin_of(l) * kTaps;
  }
  for (int l = 0; l < levels; ++l) {
    N->offG[l] = off;
    off += kC * kTaps;
  }
  for (int l = 0; l < levels; ++l) {
    N->offB[l] = off;
    off += kC;
  }
  N->nparams = off;
  auto fail_clean = [&](int s) {
    std::string msg = gd_last_error();
    gd_learned_destroy(N);
    return fail(s, msg);
  };
  int s = GD_OK;
#define ALLOC(buf, count) \
  if ((s = dalloc(buf, (size_t)(count))) != GD_OK) return fail_clean(s);
  ALLOC(N->params, N->nparams);
  ALLOC(N->grads, N->nparams);
  ALLOC(N->adam_m, N->nparams);
  ALLOC(N->adam_v, N->nparams);
  ALLOC(N->dsq, N->nlf);
  ALLOC(N->zl, N->nl[0]);
  if (N->cs) {
    ALLOC(N->xf, N->nlf);
    ALLOC(N->zf, N->nlf);
  }
  for (int l = 0; l < levels; ++l) {
    ALLOC(N->f[l], N->nl[l]);
    ALLOC(N->s[l], kC * N->nl[l]);
    for (int p = 0; p < 2; ++p) {
      ALLOC(N->x[p][l], cin_of(l) * N->nl[l]);
      ALLOC(N->a[p][l], kC * N->nl[l]);
      ALLOC(N->h[p][l], kC * N->nl[l]);
    }
    ALLOC(N->u[l], kC * N->nl[l]);
    ALLOC(N->gx[l], kC * N->nl[l]);
    ALLOC(N->d[l], kC * N->nl[l]);
    ALLOC(N->da[l], kC * N->nl[l]);
    ALLOC(N->gp[l], kC * N->nl[l]);
  }
  ALLOC(N->dred, 4096);
  ALLOC(N->zv, A->ngdofs);
  ALLOC(N->ev, A->ngdofs);
  ALLOC(N->dv, A->ngdofs);
  ALLOC(N->yv, A->ngdofs);
#undef ALLOC
  // deterministic initialisation: small convolutions (the network starts close to
  // Jacobi), gates at 0.5
  std::vector<float> p(N->nparams, 0.f);
  uint64_t rs = seed * 6364136223846793005ull + 1442695040888963407ull;
  auto rnd = [&]() {   // uniform in (-1, 1), 64-bit LCG
    rs = rs * 6364136223846793005ull + 1442695040888963407ull;
    return (float)((double)(rs >> 11) / 9007199254740992.0 * 2.0 - 1.0);
  };
  for (int l = 0; l < levels; ++l) {
    const int nw = kC * cin_of(l) * kTaps;
    for (int i = 0; i < nw; ++i) p[N->offW[l] + i] = 0.05f * rnd();
    for (int i = 0; i < kC * kTaps; ++i) p[N->offG[l] + i] = 0.05f * rnd();
  }
  cudaStream_t cs = A->test->model->ctx->stream;
  cudaError_t e = cudaMemcpyAsync(N->params.p, p.data(), sizeof(float) * N->nparams, cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaMemsetAsync(N->adam_m.p, 0, sizeof(float) * N->nparams, cs);
  if (e == cudaSuccess) e = cudaMemsetAsync(N->adam_v.p, 0, sizeof(float) * N->nparams, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  if (e != cudaSuccess) {
    fail(GD_ERR_CUDA, std::string("gd_learned_create: ") + cudaGetErrorString(e));
    return fail_clean(GD_ERR_CUDA);
  }
  *out = N;
  return GD_OK;
}

extern "C" int gd_learned_destroy(gd_learned* N) {
  if (!N) return GD_OK;
  dfreeb(N->params);
  dfreeb(N->grads);
  dfreeb(N->adam_m);
  dfreeb(N->adam_v);
  dfreeb(N->dsq);
  dfreeb(N->zl);
  dfreeb(N->xf);
  dfreeb(N->zf);
  for (int l = 0; l < kMaxLevels; ++l) {
    dfreeb(N->f[l]);
    dfreeb(N->s[l]);
    for (int p = 0; p < 2; ++p) {
      dfreeb(N->x[p][l]);
      dfreeb(N->a[p][l]);
      dfreeb(N->h[p][l]);
    }
    dfreeb(N->u[l]);
    dfreeb(N->gx[l]);
    dfreeb(N->d[l]);
    dfreeb(N->da[l]);
    dfreeb(N->gp[l]);
  }
  dfreeb(N->part);
  dfreeb(N->dred);
  dfreeb(N->zv);
  dfreeb(N->ev);
  dfreeb(N->dv);
  dfreeb(N->yv);
  delete N;
  return GD_OK;
}

extern "C" int gd_learned_num_params(const gd_learned* N, int64_t* n) {
  if (!N || !n) return fail(GD_ERR_ARG, "gd_learned_num_params: null argument");
  *n = N->nparams;
  return GD_OK;
}

extern "C" int gd_learned_levels(const gd_learned* N, int32_t* levels) {
  if (!N || !levels) return fail(GD_ERR_ARG, "gd_learned_levels: null argument");
  *levels = N->levels;
  return GD_OK;
}

extern "C" int gd_learned_flags(const gd_learned* N, int32_t* flags) {
  if (!N || !flags) return fail(GD_ERR_ARG, "gd_learned_flags: null argument");
  *flags = N->cs ? GD_LEARNED_COARSE_START : 0;
  return GD_OK;
}

extern "C" int gd_learned_get_params(const gd_learned* N, float* host) {
  if (!N || !host) return fail(GD_ERR_ARG, "gd_learned_get_params: null argument");
  cudaStream_t st = N->A->test->model->ctx->stream;
  GD_CUDA_TRY(cudaMemcpyAsync(host, N->params.p, sizeof(float) * N->nparams, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

extern "C" int gd_learned_set_params(gd_learned* N, const float* host) {
  if (!N || !host) return fail(GD_ERR_ARG, "gd_learned_set_params: null argument");
  cudaStream_t st = N->A->test->model->ctx->stream;
  GD_CUDA_TRY(cudaMemcpyAsync(N->params.p, host, sizeof(float) * N->nparams, cudaMemcpyHostToDevice, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  N->prepared = false;
  return GD_OK;
}

extern "C" int gd_learned_apply(gd_learned* N, const float* r, float* z) {
  if (!N || !r || !z) return fail(GD_ERR_ARG, "gd_learned_apply: null argument");
  cudaStream_t st = N->A->test->model->ctx->stream;
  GD_TRY(net_prepare(N, st));
  GD_TRY(net_apply_fast(N, r, z, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

// the same map through the training kernels (used to check the two paths agree)
extern "C" int gd_learned_apply_reference(gd_learned* N, const float* r, float* z) {
  if (!N || !r || !z) return fail(GD_ERR_ARG, "gd_learned_apply_reference: null argument");
  cudaStream_t st = N->A->test->model->ctx->stream;
  GD_TRY(net_prepare(N, st));
  GD_TRY(net_forward(N, r, z, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

extern "C" int gd_learned_gradient(gd_learned* N, const float* r, const float* e, int batch, double* loss,
                                   float* grads_host) {
  if (!N || !r || !e || batch < 1 || !loss) return fail(GD_ERR_ARG, "gd_learned_gradient: bad argument");
  cudaStream_t st = N->A->test->model->ctx->stream;
  const int64_t n = N->A->ngdofs;
  GD_TRY(net_prepare(N, st));
  N->prepared = false;   // gates are rebuilt once the parameters change
  GD_CUDA_TRY(cudaMemsetAsync(N->grads.p, 0, sizeof(float) * N->nparams, st));
  double total = 0.0;
  for (int b = 0; b < batch; ++b) {
    GD_TRY(net_forward(N, r + b * n, N->zv.p, st));
    double l = 0.0;
    GD_TRY(net_loss(N, N->zv.p, e + b * n, &l, N->ev.p, st));
    GD_TRY(net_backward(N, N->ev.p, st));
    total += l;
  }
  *loss = total / batch;
  if (grads_host) {
    GD_CUDA_TRY(cudaMemcpyAsync(grads_host, N->grads.p, sizeof(float) * N->nparams, cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return GD_OK;
}

extern "C" int gd_learned_train_step(gd_learned* N, const float* r, const float* e, int batch, float lr,
                                     double* loss) {
  GD_TRY(gd_learned_gradient(N, r, e, batch, loss, nullptr));
  cudaStream_t st = N->A->test->model->ctx->stream;
  ++N->adam_t;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)N->adam_t), c2 = 1.f - std::pow(b2, (float)N->adam_t);
  k_adam<<<(unsigned)((N->nparams + 255) / 256), 256, 0, st>>>((int)N->nparams, N->params.p, N->grads.p,
                                                                N->adam_m.p, N->adam_v.p, lr, b1, b2, 1e-8f, c1, c2,
                                                                1.f / batch);
  GD_CUDA_TRY(cudaGetLastError());
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  N->prepared = false;
  return GD_OK;
}

// Mixed-precision flexible CG with the network as preconditioner; Jacobi-PCG (same
// refinement) is the fallback when the learned iteration stagnates (64 inner iterations
// without halving the residual), goes non-finite or does not converge.
extern "C" int gd_solve_learned(gd_asm* A, gd_learned* N, double rtol, int maxit, double* x, int where,
                                gd_solve_stats* stats, int32_t* fallback_used) {
  if (!A || !N || N->A != A || !x) return fail(GD_ERR_ARG, "gd_solve_learned: bad argument");
  if (!A->numeric_done) return fail(GD_ERR_STATE, "gd_solve_learned: assemble the system first");
  if (A->qp_values)
    return fail(GD_ERR_UNSUPPORTED, "gd_solve_learned: the network reads cell-wise coefficients; the system was "
                                    "assembled from quadrature-point values");
  cudaStream_t st = A->test->model->ctx->stream;
  GD_TRY(net_prepare(N, st));
  MixedPrecond pc{N, apply_as_precond, apply_as_precond_lattice, N->serial};
  if (fallback_used) *fallback_used = 0;
  gd_solve_stats s1{};
  int rc = mixed_solve(A, rtol, maxit, x, where, &s1, &pc);
  if (rc == GD_ERR_STALL || rc == GD_ERR_NOTCONVERGED || rc == GD_ERR_NUMERIC) {
    gd_solve_stats s2{};
    rc = mixed_solve(A, rtol, maxit, x, where, &s2, nullptr);
    if (fallback_used) *fallback_used = 1;
    s2.iterations += s1.iterations;
    s2.seconds += s1.seconds;
    s1 = s2;
  }
  if (stats) *stats = s1;
  return rc;
}
