// mlp.cu -- the moment surrogate: a multilayer perceptron n_in -> H -> H -> n_out
// with GELU activations, trained and evaluated by hand-written kernels.
//
// Parameters live in one float32 buffer (the master copy Adam updates):
//   [W1 (H x n_in) | b1 (H) | W2 (H x H) | b2 (H) | W3 (n_out x H) | b3 (n_out)]
// Every matrix product runs on the tensor cores with bfloat16 operands and
// float32 accumulation (mma.sync m16n8k16): weights are rounded to bfloat16
// copies at the start of each call, activations are rounded when they feed the
// next product, and everything else (pre-activations, losses, gradients of the
// biases, Adam) stays float32. n_in and H must be multiples of 16; the output
// layer is padded to 16 rows internally.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "libcusna.h"
#include "saom_common.cuh"
#include "saom_launch.h"

namespace cusna {
namespace {

constexpr int kTile = 64;   // CTA tile (M and N)
constexpr int kPadK = 24;   // shared-memory row stride in bf16 (16 + 8 pad: no bank conflicts)

enum Epi : int {
  EPI_STORE = 0,     // C (fp32) = acc
  EPI_BIAS = 1,      // C = acc + bias
  EPI_BIAS_GELU = 2, // Z = acc + bias (fp32), H = gelu(Z) (bf16 and fp32)
  EPI_GELU_BWD = 3,  // D = acc * gelu'(Z) (fp32 and bf16)
};

__device__ __forceinline__ float gelu(float z) {
  return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
  const float pdf = 0.3989422804014327f * expf(-0.5f * z * z);
  return cdf + z * pdf;
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *p) {
  return *reinterpret_cast<const uint32_t *>(p);
}

// C[M x N] = A[M x K] . B[N x K]^T with bf16 A, B (row-major, leading dims lda,
// ldb in elements, both multiples of 8) and fp32 accumulation on the tensor
// cores. Requirements (checked by the host): K % 16 == 0. M and N are bounded by
// predicated loads and stores. 128 threads: four warps, each a 32 x 32 sub-tile.
template <int EPI>
__global__ void __launch_bounds__(128) gemm_bf16_tc(
    const __nv_bfloat16 *__restrict__ A, int lda, const __nv_bfloat16 *__restrict__ B, int ldb,
    int M, int N, int K, const float *__restrict__ bias, const float *__restrict__ Zin,
    float *__restrict__ Cf, __nv_bfloat16 *__restrict__ Cb, float *__restrict__ Zout, int ldc) {
  __shared__ __align__(16) __nv_bfloat16 As[kTile][kPadK];
  __shared__ __align__(16) __nv_bfloat16 Bs[kTile][kPadK];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1, g = lane >> 2, t4 = lane & 3;
  const int bm = blockIdx.y * kTile, bn = blockIdx.x * kTile;
  float acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
  const int lrow = tid >> 1, lcol = (tid & 1) * 8;
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint4 va = make_uint4(0, 0, 0, 0), vb = make_uint4(0, 0, 0, 0);
    if (bm + lrow < M) va = *reinterpret_cast<const uint4 *>(A + (size_t)(bm + lrow) * lda + k0 + lcol);
    if (bn + lrow < N) vb = *reinterpret_cast<const uint4 *>(B + (size_t)(bn + lrow) * ldb + k0 + lcol);
    *reinterpret_cast<uint4 *>(&As[lrow][lcol]) = va;
    *reinterpret_cast<uint4 *>(&Bs[lrow][lcol]) = vb;
    __syncthreads();
    uint32_t af[2][4], bf[4][2];
#pragma unroll
    for (int mi = 0; mi < 2; ++mi) {
      const int r = wm * 32 + mi * 16 + g;
      af[mi][0] = ld_pair(&As[r][2 * t4]);
      af[mi][1] = ld_pair(&As[r + 8][2 * t4]);
      af[mi][2] = ld_pair(&As[r][2 * t4 + 8]);
      af[mi][3] = ld_pair(&As[r + 8][2 * t4 + 8]);
    }
#pragma unroll
    for (int ni = 0; ni < 4; ++ni) {
      const int c = wn * 32 + ni * 8 + g;
      bf[ni][0] = ld_pair(&Bs[c][2 * t4]);
      bf[ni][1] = ld_pair(&Bs[c][2 * t4 + 8]);
    }
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
        float *d = acc[mi][ni];
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
            "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
            : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
            : "r"(af[mi][0]), "r"(af[mi][1]), "r"(af[mi][2]), "r"(af[mi][3]), "r"(bf[ni][0]),
              "r"(bf[ni][1]));
      }
    __syncthreads();
  }
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = bm + wm * 32 + mi * 16 + g + (q >= 2 ? 8 : 0);
        const int c = bn + wn * 32 + ni * 8 + 2 * t4 + (q & 1);
        if (r >= M || c >= N) continue;
        const size_t o = (size_t)r * ldc + c;
        float v = acc[mi][ni][q];
        if (EPI == EPI_STORE) {
          Cf[o] = v;
        } else if (EPI == EPI_BIAS) {
          Cf[o] = v + bias[c];
        } else if (EPI == EPI_BIAS_GELU) {
          v += bias[c];
          Zout[o] = v;
          const float h = gelu(v);
          Cb[o] = __float2bfloat16_rn(h);
        } else {  // EPI_GELU_BWD
          const float dz = v * gelu_grad(Zin[o]);
          Cf[o] = dz;
          Cb[o] = __float2bfloat16_rn(dz);
        }
      }
}

// out (cols x rows, bf16) = transpose of in (rows x cols); in may be fp32 or bf16.
template <class T>
__global__ void transpose_bf16(const T *__restrict__ in, int rows, int cols, int ldi,
                               __nv_bfloat16 *__restrict__ out, int ldo) {
  __shared__ float tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = by + y, c = bx + threadIdx.x;
    tile[y][threadIdx.x] = (r < rows && c < cols) ? (float)in[(size_t)r * ldi + c] : 0.f;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int c = bx + y, r = by + threadIdx.x;
    if (c < cols && r < rows) out[(size_t)c * ldo + r] = __float2bfloat16_rn(tile[threadIdx.x][y]);
  }
}

__global__ void to_bf16(const float *__restrict__ in, size_t n, __nv_bfloat16 *__restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(in[i]);
}

// out (B x cols, bf16) = rows sel[0..B) of in (fp32, cols per row); sel NULL
// means rows 0..B.
__global__ void gather_bf16(const float *__restrict__ in, const int32_t *__restrict__ sel, int B,
                            int cols, __nv_bfloat16 *__restrict__ out) {
  const size_t n = (size_t)B * cols;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    const size_t src = sel ? (size_t)sel[r] : (size_t)r;
    out[i] = __float2bfloat16_rn(in[src * cols + c]);
  }
}

// rows x cols fp32 matrix (ld) -> padded bf16 (rows_pad x cols_pad), zeros outside
__global__ void pad_bf16(const float *__restrict__ in, int rows, int cols, int ldi, int rows_pad,
                         int cols_pad, __nv_bfloat16 *__restrict__ out) {
  const size_t n = (size_t)rows_pad * cols_pad;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols_pad), c = (int)(i % cols_pad);
    out[i] = __float2bfloat16_rn((r < rows && c < cols) ? in[(size_t)r * ldi + c] : 0.f);
  }
}

// Mean-squared-error loss over the n_out real columns of Y (B x ldy) against
// rows sel[0..B) of T (NULL: rows 0..B); dY (B x ldy, fp32 and bf16) =
// 2 (Y - T) / (B n_out), zero in the padding; loss[0] += the loss.
__global__ void mse_grad(const float *__restrict__ Y, int ldy, const float *__restrict__ T,
                         const int32_t *__restrict__ sel, int B, int n_out,
                         float *__restrict__ dY, __nv_bfloat16 *__restrict__ dYb,
                         float *__restrict__ loss) {
  float part = 0.f;
  const float scale = 2.f / ((float)B * n_out);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B * ldy; i += gridDim.x * blockDim.x) {
    const int r = i / ldy, c = i % ldy;
    float d = 0.f;
    if (c < n_out) {
      const size_t tr = sel ? (size_t)sel[r] : (size_t)r;
      const float e = Y[i] - T[tr * n_out + c];
      part += e * e;
      d = scale * e;
    }
    dY[i] = d;
    dYb[i] = __float2bfloat16_rn(d);
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, part / ((float)B * n_out));
}

// out[c] = sum over the rows of D (rows x ld) of column c, c < cols. One CTA
// of 32 x 32 threads per 32 columns: thread (x, y) sums rows y, y + 32, ...
// in order, then the 32 partial sums are added in a fixed order
// (deterministic, no atomics).
__global__ void __launch_bounds__(1024) col_sum(const float *__restrict__ D, int rows, int cols,
                                                int ld, float *__restrict__ out) {
  __shared__ float part[32][33];
  const int c = blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (c < cols)
    for (int r = threadIdx.y; r < rows; r += 32) s += D[(size_t)r * ld + c];
  part[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && c < cols) {
    float t = 0.f;
    for (int y = 0; y < 32; ++y) t += part[y][threadIdx.x];
    out[c] = t;
  }
}

// Adam (Kingma & Ba 2015) with bias correction, in place on fp32 buffers.
__global__ void adam_step(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                          float c1, float c2) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Device-side Adam bookkeeping, so that a sequence of steps has no host
// arguments that change from step to step (and can be replayed as a graph).
__global__ void adam_bump(cusna_adam_hyper *h) {
  const int step = h->step + 1;
  h->step = step;
  h->c1 = 1.f - powf(h->beta1, (float)step);
  h->c2 = 1.f - powf(h->beta2, (float)step);
}

__global__ void adam_step_dev(float *__restrict__ p, const float *__restrict__ g,
                              float *__restrict__ m, float *__restrict__ v, size_t n,
                              const cusna_adam_hyper *__restrict__ h) {
  const float lr = h->lr, b1 = h->beta1, b2 = h->beta2, eps = h->eps, c1 = h->c1, c2 = h->c2;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Gaussian initialisation N(0, scale^2) from the Philox generator (Box-Muller).
__global__ void init_normal(float *p, size_t n, float scale, uint32_t k0, uint32_t k1, uint32_t tag) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t r[4];
    philox10((uint32_t)i, tag, 7u, 0u, k0, k1, r);
    const float u1 = ((float)r[0] + 0.5f) * 2.3283064365386963e-10f;
    const float u2 = ((float)r[1] + 0.5f) * 2.3283064365386963e-10f;
    p[i] = scale * sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
  }
}

// Forward-mode derivative of the network outputs with respect to the first
// n_wrt inputs, one CTA per point: t1 = W1[:, i] gelu'(z1), t2 = W2 t1
// gelu'(z2), J[:, i] = W3 t2 (float32 throughout, from the pre-activations of a
// forward pass).
__global__ void jacobian_fwd(const float *__restrict__ P, const float *__restrict__ Z1,
                             const float *__restrict__ Z2, int n_in, int H, int n_out, int n_wrt,
                             float *__restrict__ J) {
  extern __shared__ float sh[];
  float *t1 = sh, *t2 = sh + H;
  const int b = blockIdx.x;
  const float *W1 = P, *W2 = P + (size_t)H * n_in + H, *W3 = W2 + (size_t)H * H + H;
  for (int i = 0; i < n_wrt; ++i) {
    for (int h = threadIdx.x; h < H; h += blockDim.x)
      t1[h] = W1[(size_t)h * n_in + i] * gelu_grad(Z1[(size_t)b * H + h]);
    __syncthreads();
    for (int h = threadIdx.x; h < H; h += blockDim.x) {
      float s = 0.f;
      for (int q = 0; q < H; ++q) s += W2[(size_t)h * H + q] * t1[q];
      t2[h] = s * gelu_grad(Z2[(size_t)b * H + h]);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < n_out; o += blockDim.x) {
      float s = 0.f;
      for (int q = 0; q < H; ++q) s += W3[(size_t)o * H + q] * t2[q];
      J[((size_t)b * n_out + o) * n_wrt + i] = s;
    }
    __syncthreads();
  }
}

// ---- workspace layout ------------------------------------------------------
struct Ws {
  __nv_bfloat16 *w1b, *w2b, *w3b, *w2t, *w3t, *xb, *xt, *h1b, *h1t, *h2b, *h2t, *dyb, *dyt,
      *dz2b, *dz2t, *dz1b, *dz1t;
  float *z1, *z2, *y, *dy, *dz2, *dz1, *loss;
};

constexpr int kOutPad = 16;

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t ws_layout(int n_in, int H, int B, unsigned char *base, Ws *w) {
  const int O = kOutPad;
  size_t off = 0;
  auto bf = [&](__nv_bfloat16 **p, size_t cnt) {
    if (base) *p = (__nv_bfloat16 *)(base + off);
    off = align256(off + cnt * 2);
  };
  auto f32 = [&](float **p, size_t cnt) {
    if (base) *p = (float *)(base + off);
    off = align256(off + cnt * 4);
  };
  Ws d{};
  Ws &x = w ? *w : d;
  bf(&x.w1b, (size_t)H * n_in); bf(&x.w2b, (size_t)H * H); bf(&x.w3b, (size_t)O * H);
  bf(&x.w2t, (size_t)H * H); bf(&x.w3t, (size_t)H * O);
  bf(&x.xb, (size_t)B * n_in); bf(&x.xt, (size_t)n_in * B);
  bf(&x.h1b, (size_t)B * H); bf(&x.h1t, (size_t)H * B);
  bf(&x.h2b, (size_t)B * H); bf(&x.h2t, (size_t)H * B);
  bf(&x.dyb, (size_t)B * O); bf(&x.dyt, (size_t)O * B);
  bf(&x.dz2b, (size_t)B * H); bf(&x.dz2t, (size_t)H * B);
  bf(&x.dz1b, (size_t)B * H); bf(&x.dz1t, (size_t)H * B);
  f32(&x.z1, (size_t)B * H); f32(&x.z2, (size_t)B * H); f32(&x.y, (size_t)B * O);
  f32(&x.dy, (size_t)B * O); f32(&x.dz2, (size_t)B * H); f32(&x.dz1, (size_t)B * H);
  f32(&x.loss, 4);
  return off;
}

int blocks_for(size_t n) {
  size_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 2048 ? 2048 : b));
}

template <int EPI>
cudaError_t gemm(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N,
                 int K, const float *bias, const float *Zin, float *Cf, __nv_bfloat16 *Cb,
                 float *Zout, int ldc, cudaStream_t st) {
  dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
  gemm_bf16_tc<EPI><<<grid, 128, 0, st>>>(A, lda, B, ldb, M, N, K, bias, Zin, Cf, Cb, Zout, ldc);
  return cudaGetLastError();
}

template <class T>
cudaError_t transpose(const T *in, int rows, int cols, int ldi, __nv_bfloat16 *out, int ldo,
                      cudaStream_t st) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  transpose_bf16<T><<<grid, block, 0, st>>>(in, rows, cols, ldi, out, ldo);
  return cudaGetLastError();
}

bool dims_ok(int n_in, int H, int n_out) {
  return n_in > 0 && n_in % 16 == 0 && H > 0 && H % 16 == 0 && H <= 4096 && n_out > 0 &&
         n_out <= kOutPad;
}

#define MCU(call)                                                         \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) {                                              \
      set_last_error(cudaGetErrorString(e_));                             \
      return CUSNA_ERR_CUDA;                                              \
    }                                                                     \
  } while (0)

// Shape and workspace checks shared by the entry points; training batches
// must be multiples of 16 (the batch is the reduction dimension of the
// weight-gradient products).
cusna_status check_call(int n_in, int H, int n_out, int B, bool training, size_t work_bytes) {
  if (!dims_ok(n_in, H, n_out) || B < 1 || (training && B % 16 != 0)) {
    set_last_error("mlp: n_in and hidden must be positive multiples of 16, n_out in 1..16, "
                   "training batches a multiple of 16");
    return CUSNA_ERR_SHAPE;
  }
  if (ws_layout(n_in, H, B, nullptr, nullptr) > work_bytes) {
    set_last_error("mlp: workspace smaller than cusna_mlp_workspace_bytes for this batch");
    return CUSNA_ERR_SHAPE;
  }
  return CUSNA_OK;
}

// bf16 weight copies (and the transposed W2, W3 the backward pass reads)
cusna_status refresh_weights(const float *P, int n_in, int H, int n_out, const Ws &w, cudaStream_t st) {
  const float *W1 = P, *W2 = P + (size_t)H * n_in + H, *W3 = W2 + (size_t)H * H + H;
  to_bf16<<<blocks_for((size_t)H * n_in), 256, 0, st>>>(W1, (size_t)H * n_in, w.w1b);
  to_bf16<<<blocks_for((size_t)H * H), 256, 0, st>>>(W2, (size_t)H * H, w.w2b);
  pad_bf16<<<blocks_for((size_t)kOutPad * H), 256, 0, st>>>(W3, n_out, H, H, kOutPad, H, w.w3b);
  MCU(cudaGetLastError());
  MCU(transpose(W2, H, H, H, w.w2t, H, st));
  MCU(transpose(w.w3b, kOutPad, H, H, w.w3t, kOutPad, st));
  return CUSNA_OK;
}

cusna_status forward(const float *P, const float *X, const int32_t *sel, int n_in, int H,
                     int n_out, int B, const Ws &w, cudaStream_t st) {
  const float *b1 = P + (size_t)H * n_in, *b2 = b1 + H + (size_t)H * H, *b3 = b2 + H + (size_t)n_out * H;
  gather_bf16<<<blocks_for((size_t)B * n_in), 256, 0, st>>>(X, sel, B, n_in, w.xb);
  MCU(cudaGetLastError());
  MCU(gemm<EPI_BIAS_GELU>(w.xb, n_in, w.w1b, n_in, B, H, n_in, b1, nullptr, nullptr, w.h1b, w.z1, H, st));
  MCU(gemm<EPI_BIAS_GELU>(w.h1b, H, w.w2b, H, B, H, H, b2, nullptr, nullptr, w.h2b, w.z2, H, st));
  MCU(gemm<EPI_BIAS>(w.h2b, H, w.w3b, H, B, n_out, H, b3, nullptr, w.y, nullptr, nullptr, kOutPad, st));
  return CUSNA_OK;
}

// Gradient of the mean-squared error into G (same layout as P); w.loss
// receives the loss.
cusna_status backward(const float *T, const int32_t *sel, int n_in, int H, int n_out, int B,
                      float *G, const Ws &w, cudaStream_t st) {
  float *gW1 = G, *gb1 = G + (size_t)H * n_in, *gW2 = gb1 + H, *gb2 = gW2 + (size_t)H * H,
        *gW3 = gb2 + H, *gb3 = gW3 + (size_t)n_out * H;
  const int O = kOutPad;
  const dim3 cs(32, 32);
  MCU(cudaMemsetAsync(w.loss, 0, sizeof(float), st));
  mse_grad<<<blocks_for((size_t)B * O), 256, 0, st>>>(w.y, O, T, sel, B, n_out, w.dy, w.dyb, w.loss);
  MCU(cudaGetLastError());
  // layer 3: gW3 = dY^T H2 (n_out x H), dZ2 = (dY W3) * gelu'(Z2)
  MCU(transpose(w.dyb, B, O, O, w.dyt, B, st));
  MCU(transpose(w.h2b, B, H, H, w.h2t, B, st));
  MCU(gemm<EPI_STORE>(w.dyt, B, w.h2t, B, n_out, H, B, nullptr, nullptr, gW3, nullptr, nullptr, H, st));
  col_sum<<<(n_out + 31) / 32, cs, 0, st>>>(w.dy, B, n_out, O, gb3);
  MCU(gemm<EPI_GELU_BWD>(w.dyb, O, w.w3t, O, B, H, O, nullptr, w.z2, w.dz2, w.dz2b, nullptr, H, st));
  // layer 2: gW2 = dZ2^T H1, dZ1 = (dZ2 W2) * gelu'(Z1)
  MCU(transpose(w.dz2b, B, H, H, w.dz2t, B, st));
  MCU(transpose(w.h1b, B, H, H, w.h1t, B, st));
  MCU(gemm<EPI_STORE>(w.dz2t, B, w.h1t, B, H, H, B, nullptr, nullptr, gW2, nullptr, nullptr, H, st));
  col_sum<<<(H + 31) / 32, cs, 0, st>>>(w.dz2, B, H, H, gb2);
  MCU(gemm<EPI_GELU_BWD>(w.dz2b, H, w.w2t, H, B, H, H, nullptr, w.z1, w.dz1, w.dz1b, nullptr, H, st));
  // layer 1: gW1 = dZ1^T X
  MCU(transpose(w.dz1b, B, H, H, w.dz1t, B, st));
  MCU(transpose(w.xb, B, n_in, n_in, w.xt, B, st));
  MCU(gemm<EPI_STORE>(w.dz1t, B, w.xt, B, H, n_in, B, nullptr, nullptr, gW1, nullptr, nullptr, n_in, st));
  col_sum<<<(H + 31) / 32, cs, 0, st>>>(w.dz1, B, H, H, gb1);
  MCU(cudaGetLastError());
  return CUSNA_OK;
}

cusna_status grad_impl(const float *params, const float *x, const float *t, const int32_t *sel,
                       int B, float *grad, float *loss, void *work, size_t work_bytes, int n_in,
                       int H, int n_out, cudaStream_t st) {
  if (!params || !x || !t || !grad || !work) return CUSNA_ERR_NULL_ARG;
  cusna_status s = check_call(n_in, H, n_out, B, true, work_bytes);
  if (s != CUSNA_OK) return s;
  Ws w{};
  ws_layout(n_in, H, B, (unsigned char *)work, &w);
  if ((s = refresh_weights(params, n_in, H, n_out, w, st)) != CUSNA_OK) return s;
  if ((s = forward(params, x, sel, n_in, H, n_out, B, w, st)) != CUSNA_OK) return s;
  if ((s = backward(t, sel, n_in, H, n_out, B, grad, w, st)) != CUSNA_OK) return s;
  if (loss) MCU(cudaMemcpyAsync(loss, w.loss, sizeof(float), cudaMemcpyDeviceToDevice, st));
  return CUSNA_OK;
}

struct TrainArgs {
  float *params, *grad, *m, *v;
  const float *x, *t;
  const int32_t *rows;
  int B, n_steps;
  cusna_adam_hyper *hyper;
  float *losses;
  void *work;
  size_t work_bytes;
  int n_in, H, n_out;
  bool operator==(const TrainArgs &o) const { return std::memcmp(this, &o, sizeof(*this)) == 0; }
};

// n_steps minibatch steps: step s uses rows[s*B .. (s+1)*B) (rows NULL: rows
// 0..B every step), then Adam with the device-side step counter.
cusna_status train_steps_impl(const TrainArgs &a, cudaStream_t st) {
  const size_t n = (size_t)a.H * a.n_in + a.H + (size_t)a.H * a.H + a.H + (size_t)a.n_out * a.H + a.n_out;
  for (int s = 0; s < a.n_steps; ++s) {
    cusna_status r = grad_impl(a.params, a.x, a.t, a.rows ? a.rows + (size_t)s * a.B : nullptr, a.B,
                               a.grad, a.losses ? a.losses + s : nullptr, a.work, a.work_bytes,
                               a.n_in, a.H, a.n_out, st);
    if (r != CUSNA_OK) return r;
    adam_bump<<<1, 1, 0, st>>>(a.hyper);
    adam_step_dev<<<blocks_for(n), 256, 0, st>>>(a.params, a.grad, a.m, a.v, n, a.hyper);
    MCU(cudaGetLastError());
  }
  return CUSNA_OK;
}

// Instantiated graphs of train_steps_impl, one per distinct argument set
// (pointers and sizes; the values behind the pointers may change between
// replays). A few entries, oldest evicted first.
struct GraphEntry {
  int device;
  TrainArgs args;
  cudaGraphExec_t exec;
};
constexpr size_t kMaxGraphs = 8;
std::mutex g_graph_mu;
std::vector<GraphEntry> g_graphs;

cusna_status replay_train_graph(const TrainArgs &a, cudaStream_t st) {
  int dev = 0;
  MCU(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_graph_mu);
  for (auto &e : g_graphs)
    if (e.device == dev && e.args == a) {
      MCU(cudaGraphLaunch(e.exec, st));
      return CUSNA_OK;
    }
  cudaStream_t cap = nullptr;
  MCU(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaError_t e0 = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e0 != cudaSuccess) {
    cudaStreamDestroy(cap);
    set_last_error(cudaGetErrorString(e0));
    return CUSNA_ERR_CUDA;
  }
  cusna_status r = train_steps_impl(a, cap);
  cudaGraph_t graph = nullptr;
  cudaError_t e1 = cudaStreamEndCapture(cap, &graph);   // ends the capture on every path
  cudaStreamDestroy(cap);
  if (r != CUSNA_OK || e1 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    if (r == CUSNA_OK) set_last_error(cudaGetErrorString(e1));
    return r != CUSNA_OK ? r : CUSNA_ERR_CUDA;
  }
  cudaGraphExec_t exec = nullptr;
  cudaError_t e2 = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e2 != cudaSuccess) {
    set_last_error(cudaGetErrorString(e2));
    return CUSNA_ERR_CUDA;
  }
  if (g_graphs.size() >= kMaxGraphs) {
    cudaGraphExecDestroy(g_graphs.front().exec);
    g_graphs.erase(g_graphs.begin());
  }
  g_graphs.push_back(GraphEntry{dev, a, exec});
  MCU(cudaGraphLaunch(exec, st));
  return CUSNA_OK;
}

}  // namespace
}  // namespace cusna

using namespace cusna;

extern "C" {

CUSNA_API size_t cusna_mlp_param_count(int32_t n_in, int32_t hidden, int32_t n_out) {
  return (size_t)hidden * n_in + hidden + (size_t)hidden * hidden + hidden + (size_t)n_out * hidden + n_out;
}

CUSNA_API size_t cusna_mlp_workspace_bytes(int32_t n_in, int32_t hidden, int32_t n_out,
                                           int32_t batch) {
  (void)n_out;
  if (n_in < 1 || hidden < 1 || batch < 1) return 0;
  return ws_layout(n_in, hidden, batch, nullptr, nullptr);
}

CUSNA_API cusna_status cusna_mlp_init(float *params, int32_t n_in, int32_t hidden, int32_t n_out,
                                      uint64_t seed, void *stream) {
  if (!params) return CUSNA_ERR_NULL_ARG;
  if (!dims_ok(n_in, hidden, n_out)) return CUSNA_ERR_SHAPE;
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  float *W1 = params, *b1 = W1 + (size_t)hidden * n_in, *W2 = b1 + hidden, *b2 = W2 + (size_t)hidden * hidden,
        *W3 = b2 + hidden, *b3 = W3 + (size_t)n_out * hidden;
  // He initialisation for the GELU layers; the output layer and every bias
  // start at zero, so an untrained network predicts exactly zero
  init_normal<<<blocks_for((size_t)hidden * n_in), 256, 0, st>>>(W1, (size_t)hidden * n_in, sqrtf(2.f / n_in), k0, k1, 1);
  init_normal<<<blocks_for((size_t)hidden * hidden), 256, 0, st>>>(W2, (size_t)hidden * hidden, sqrtf(2.f / hidden), k0, k1, 2);
  MCU(cudaGetLastError());
  MCU(cudaMemsetAsync(W3, 0, (size_t)n_out * hidden * 4, st));
  MCU(cudaMemsetAsync(b1, 0, hidden * 4, st));
  MCU(cudaMemsetAsync(b2, 0, hidden * 4, st));
  MCU(cudaMemsetAsync(b3, 0, n_out * 4, st));
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_mlp_forward(const float *params, const float *x, int32_t batch,
                                         float *y, void *work, size_t work_bytes, int32_t n_in,
                                         int32_t hidden, int32_t n_out, void *stream) {
  if (!params || !x || !y || !work) return CUSNA_ERR_NULL_ARG;
  cusna_status s = check_call(n_in, hidden, n_out, batch, false, work_bytes);
  if (s != CUSNA_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  Ws w{};
  ws_layout(n_in, hidden, batch, (unsigned char *)work, &w);
  if ((s = refresh_weights(params, n_in, hidden, n_out, w, st)) != CUSNA_OK) return s;
  if ((s = forward(params, x, nullptr, n_in, hidden, n_out, batch, w, st)) != CUSNA_OK) return s;
  MCU(cudaMemcpy2DAsync(y, (size_t)n_out * 4, w.y, (size_t)kOutPad * 4, (size_t)n_out * 4, batch,
                        cudaMemcpyDeviceToDevice, st));
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_mlp_grad(const float *params, const float *x, const float *t,
                                      const int32_t *rows, int32_t batch, float *grad,
                                      float *loss, void *work, size_t work_bytes, int32_t n_in,
                                      int32_t hidden, int32_t n_out, void *stream) {
  return grad_impl(params, x, t, rows, batch, grad, loss, work, work_bytes, n_in, hidden, n_out,
                   (cudaStream_t)stream);
}

CUSNA_API cusna_status cusna_mlp_train_step(float *params, float *grad, float *adam_m,
                                            float *adam_v, const float *x, const float *t,
                                            const int32_t *rows, int32_t batch, int32_t step,
                                            float lr, float beta1, float beta2, float eps,
                                            float *loss, void *work, size_t work_bytes,
                                            int32_t n_in, int32_t hidden, int32_t n_out,
                                            void *stream) {
  if (!adam_m || !adam_v) return CUSNA_ERR_NULL_ARG;
  if (step < 1) return CUSNA_ERR_SHAPE;
  cudaStream_t st = (cudaStream_t)stream;
  cusna_status s = grad_impl(params, x, t, rows, batch, grad, loss, work, work_bytes, n_in,
                             hidden, n_out, st);
  if (s != CUSNA_OK) return s;
  const size_t n = cusna_mlp_param_count(n_in, hidden, n_out);
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  adam_step<<<blocks_for(n), 256, 0, st>>>(params, grad, adam_m, adam_v, n, lr, beta1, beta2, eps,
                                           c1, c2);
  MCU(cudaGetLastError());
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_mlp_train_steps(float *params, float *grad, float *adam_m,
                                             float *adam_v, const float *x, const float *t,
                                             const int32_t *rows, int32_t batch, int32_t n_steps,
                                             cusna_adam_hyper *hyper, float *losses, void *work,
                                             size_t work_bytes, int32_t n_in, int32_t hidden,
                                             int32_t n_out, int32_t use_graph, void *stream) {
  if (!params || !grad || !adam_m || !adam_v || !x || !t || !hyper || !work)
    return CUSNA_ERR_NULL_ARG;
  if (n_steps < 1 || n_steps > (1 << 16)) return CUSNA_ERR_SHAPE;
  cusna_status s = check_call(n_in, hidden, n_out, batch, true, work_bytes);
  if (s != CUSNA_OK) return s;
  TrainArgs a;
  std::memset(&a, 0, sizeof(a));   // padding too: graphs are looked up by memcmp
  a.params = params; a.grad = grad; a.m = adam_m; a.v = adam_v; a.x = x; a.t = t; a.rows = rows;
  a.B = batch; a.n_steps = n_steps; a.hyper = hyper; a.losses = losses; a.work = work;
  a.work_bytes = work_bytes; a.n_in = n_in; a.H = hidden; a.n_out = n_out;
  cudaStream_t st = (cudaStream_t)stream;
  NvtxRange r("cusna_mlp_train_steps");
  return use_graph ? replay_train_graph(a, st) : train_steps_impl(a, st);
}

CUSNA_API cusna_status cusna_mlp_jacobian(const float *params, const float *x, int32_t batch,
                                          int32_t n_wrt, float *y, float *J, void *work,
                                          size_t work_bytes, int32_t n_in, int32_t hidden,
                                          int32_t n_out, void *stream) {
  if (!J) return CUSNA_ERR_NULL_ARG;
  if (n_wrt < 1 || n_wrt > n_in) return CUSNA_ERR_SHAPE;
  cusna_status s = cusna_mlp_forward(params, x, batch, y, work, work_bytes, n_in, hidden, n_out, stream);
  if (s != CUSNA_OK) return s;
  Ws w{};
  ws_layout(n_in, hidden, batch, (unsigned char *)work, &w);
  jacobian_fwd<<<batch, 128, 2 * hidden * sizeof(float), (cudaStream_t)stream>>>(
      params, w.z1, w.z2, n_in, hidden, n_out, n_wrt, J);
  MCU(cudaGetLastError());
  return CUSNA_OK;
}

}  // extern "C"
