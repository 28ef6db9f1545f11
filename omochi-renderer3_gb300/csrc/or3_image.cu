// or3_image.cu -- image output and input on the device: the reference savers'
// 8-bit conversion, RGBE encode/decode, and the environment map's sampling CDF.
//
//   8-bit   FileSaver::CopyColorArrayToImage (src/tools/FileSaver.h:49-120):
//           clamp to [0, 1], gamma pow(x, 1/2.2) (Utils::GammaRev,
//           src/tools/Utils.h:99-101); then Utils::ToRgb (:107-109),
//           (int)(v * 255 + 0.5), as ImageHandler::SaveToPngFile writes it
//           (src/tools/ImageHandler.cpp:133-155).  With gamma the byte is a
//           monotone step function of the clamped value, so the kernel looks
//           it up among 255 thresholds found once on the host with the host's
//           own pow: every byte equals what the reference's conversion gives
//           on the same double, without a transcendental on the device.
//   RGBE    HDRImage::Color2RGBE / RGBE2Color (src/tools/HDRImage.h:10-38),
//           in the same float/double operations (all exact or correctly
//           rounded, so the bytes match).
//   env CDF one block per row (weights max(r,g,b) * sin(theta) and the row's
//           running sums in double), one block for the rows' marginal; the
//           same tables the host build produced, in a fixed summation order.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "or3.h"
#include "or3_internal.h"
#include "or3_kernels.cuh"

namespace or3 {
namespace {

__constant__ double c_gamma_thr[256];  // smallest clamped value whose gamma byte is >= k (k >= 1)

int host_to8(double c) { return (int)(std::pow(c, 1.0 / 2.2) * 255 + 0.5); }

// thresholds by bisection over the bit patterns of doubles in [0, 1]
const std::vector<double> &gamma_thresholds() {
  static std::vector<double> th;
  static std::once_flag once;
  std::call_once(once, [] {
    th.assign(256, 0.0);
    for (int k = 1; k < 256; k++) {
      uint64_t lo = 0, hi;  // code(lo) < k <= code(hi)
      const double one = 1.0;
      std::memcpy(&hi, &one, 8);
      while (hi - lo > 1) {
        const uint64_t mid = lo + (hi - lo) / 2;
        double m;
        std::memcpy(&m, &mid, 8);
        if (host_to8(m) >= k) hi = mid;
        else lo = mid;
      }
      std::memcpy(&th[k], &hi, 8);
    }
  });
  return th;
}

std::mutex g_thr_mu;
bool g_thr_done[64] = {};

__device__ __forceinline__ double clamp01(double x) { return x > 0.0 ? (x < 1.0 ? x : 1.0) : 0.0; }  // NaN -> 0

__global__ void k_encode_rgb8(size_t nvals, const double *in, int gamma, uint8_t *out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvals) return;
  const double v = clamp01(in[i]);
  int code;
  if (gamma) {
    int lo = 0;  // largest k with thr[k] <= v (thr[0] = 0)
#pragma unroll
    for (int step = 128; step > 0; step >>= 1)
      if (lo + step < 256 && c_gamma_thr[lo + step] <= v) lo += step;
    code = lo;
  } else {
    code = (int)(v * 255 + 0.5);
  }
  out[i] = (uint8_t)code;
}

__global__ void k_encode_rgbe(size_t n, const double *in, uint8_t *out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double r = in[3 * i], g = in[3 * i + 1], b = in[3 * i + 2];
  float v = (float)fmax(fmax(r, g), b);
  uchar4 o = make_uchar4(0, 0, 0, 0);
  if (!((double)v < 1e-32)) {
    int e;
    v = __fdiv_rn(__fmul_rn(frexpf(v, &e), 256.0f), v);
    o = make_uchar4((uint8_t)(r * (double)v), (uint8_t)(g * (double)v), (uint8_t)(b * (double)v), (uint8_t)(e + 128));
  }
  reinterpret_cast<uchar4 *>(out)[i] = o;
}

__global__ void k_decode_rgbe(size_t n, const uint8_t *in, float *out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uchar4 c = reinterpret_cast<const uchar4 *>(in)[i];
  float r = 0.f, g = 0.f, b = 0.f;
  if (c.w) {
    const float f = ldexpf(1.0f, (int)c.w - (128 + 8));
    r = __fmul_rn((float)c.x, f);
    g = __fmul_rn((float)c.y, f);
    b = __fmul_rn((float)c.z, f);
  }
  out[3 * i] = r;
  out[3 * i + 1] = g;
  out[3 * i + 2] = b;
}

// exclusive block scan of one double per thread (blockDim.x a multiple of 32,
// at most 1024); *total receives the block's sum (shared, read after return)
__device__ double block_exclusive_scan(double v, double *total) {
  __shared__ double ws[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = 0;
    const int nw = blockDim.x / 32;
    for (int w = 0; w < nw; w++) {
      const double x = ws[w];
      ws[w] = acc;
      acc += x;
    }
    *total = acc;
  }
  __syncthreads();
  const double r = ws[warp] + incl - v;
  __syncthreads();
  return r;
}

__device__ __forceinline__ double env_weight(const float *p, double st) {
  const float mx = fmaxf(p[0], fmaxf(p[1], p[2]));
  return (mx > 0.f ? (double)mx : 0.0) * st;
}

// one block per row: conditional CDF of the row, and the row's total
__global__ void __launch_bounds__(256) k_env_rows(const float *env, uint32_t W, uint32_t H, float *cond,
                                                  double *rows) {
  __shared__ double tot;
  const uint32_t i = blockIdx.x;
  const double st = sin(3.14159265358979323846264338327950288 * (i + 0.5) / H);
  const float *row = env + 3 * (size_t)i * W;
  const uint32_t per = (W + blockDim.x - 1) / blockDim.x, j0 = threadIdx.x * per;
  double s = 0;
  for (uint32_t k = 0; k < per && j0 + k < W; k++) s += env_weight(row + 3 * (j0 + k), st);
  double run = block_exclusive_scan(s, &tot);
  const double total = tot;
  for (uint32_t k = 0; k < per && j0 + k < W; k++) {
    const uint32_t j = j0 + k;
    run += env_weight(row + 3 * j, st);
    cond[(size_t)i * W + j] = j + 1 == W ? 1.0f : total > 0 ? (float)(run / total) : (float)((j + 1.0) / W);
  }
  if (threadIdx.x == 0) rows[i] = total;
}

// one block: marginal CDF over the rows; rows[H] receives the map's total
__global__ void __launch_bounds__(1024) k_env_marg(uint32_t H, double *rows, float *marg) {
  __shared__ double tot;
  const uint32_t per = (H + blockDim.x - 1) / blockDim.x, i0 = threadIdx.x * per;
  double s = 0;
  for (uint32_t k = 0; k < per && i0 + k < H; k++) s += rows[i0 + k];
  double run = block_exclusive_scan(s, &tot);
  const double total = tot;
  for (uint32_t k = 0; k < per && i0 + k < H; k++) {
    const uint32_t i = i0 + k;
    run += rows[i];
    marg[i] = i + 1 == H ? 1.0f : total > 0 ? (float)(run / total) : (float)((i + 1.0) / H);
  }
  __syncthreads();
  if (threadIdx.x == 0) rows[H] = total;
}

// Guide tables of the CDFs above: thread k of row r stores the first index
// whose CDF value exceeds k / n (n - 1 if none), k = 0..n; one block per row.
__global__ void __launch_bounds__(256) k_env_guide(const float *cdf, uint32_t n, uint32_t *guide) {
  const float *c = cdf + (size_t)blockIdx.x * n;
  uint32_t *g = guide + (size_t)blockIdx.x * (n + 1);
  for (uint32_t k = threadIdx.x; k <= n; k += blockDim.x) {
    const float t = (float)k / (float)n;
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (c[mid] > t) hi = mid;
      else lo = mid + 1;
    }
    g[k] = lo;
  }
}

}  // namespace

int ensure_gamma_table(int device) {
  if (device < 0 || device >= 64) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_thr_mu);
  if (g_thr_done[device]) return 0;
  const std::vector<double> &th = gamma_thresholds();
  const cudaError_t e = cudaMemcpyToSymbol(c_gamma_thr, th.data(), 256 * sizeof(double));
  if (e != cudaSuccess) return (int)e;
  g_thr_done[device] = true;
  return 0;
}

void launch_encode_rgb8(const double *in, size_t nvals, int gamma, uint8_t *out, cudaStream_t st) {
  if (nvals) k_encode_rgb8<<<(unsigned)((nvals + 255) / 256), 256, 0, st>>>(nvals, in, gamma, out);
}

void launch_encode_rgbe(const double *in, size_t npix, uint8_t *out, cudaStream_t st) {
  if (npix) k_encode_rgbe<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(npix, in, out);
}

void launch_decode_rgbe(const uint8_t *in, size_t npix, float *out, cudaStream_t st) {
  if (npix) k_decode_rgbe<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(npix, in, out);
}

void launch_env_cdf(const float *env, uint32_t W, uint32_t H, float *marg, float *cond, double *rows,
                    uint32_t *gmarg, uint32_t *gcond, cudaStream_t st) {
  k_env_rows<<<H, 256, 0, st>>>(env, W, H, cond, rows);
  k_env_marg<<<1, 1024, 0, st>>>(H, rows, marg);
  k_env_guide<<<H, 256, 0, st>>>(cond, W, gcond);
  k_env_guide<<<1, 256, 0, st>>>(marg, H, gmarg);
}

}  // namespace or3

using namespace or3;

namespace {

// host data -> device -> kernel -> host, on the context's stream
template <class In, class Out, class Launch>
int transcode(or3_context *ctx, const In *in, size_t nin, Out *out, size_t nout, Launch launch) {
  In *din = nullptr;
  Out *dout = nullptr;
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMalloc(&din, std::max<size_t>(nin, 1) * sizeof(In));
  if (e == cudaSuccess) e = cudaMalloc(&dout, std::max<size_t>(nout, 1) * sizeof(Out));
  if (e == cudaSuccess) e = cudaMemcpyAsync(din, in, nin * sizeof(In), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    launch(din, dout, st);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, nout * sizeof(Out), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(din);
  cudaFree(dout);
  if (e != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "image conversion: %s", cudaGetErrorString(e));
  return OR3_OK;
}

// the last frame on the device, encoded by `launch` into `per` bytes per pixel
template <class Launch>
int frame_bytes(or3_context *ctx, uint8_t *out, size_t capacity, int32_t *samples, size_t per, Launch launch) {
  size_t nd = 0;
  {
    std::lock_guard<std::mutex> lk(ctx->frame_mu);
    if (samples) *samples = ctx->frame_samples;
    nd = ctx->front_doubles;
  }
  if (nd == 0) return fail(ctx, OR3_ERR_NOT_FOUND, "no frame rendered yet");
  const size_t npix = nd / 3;
  if (!out || capacity < per * npix) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "frame needs %zu bytes", per * npix);
  cudaSetDevice(ctx->device);
  uint8_t *d = nullptr;
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMalloc(&d, per * npix);
  if (e == cudaSuccess) {
    launch(ctx->frame_dev, npix, d, st);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, per * npix, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d);
  if (e != cudaSuccess) return fail(ctx, OR3_ERR_CUDA, "frame encode: %s", cudaGetErrorString(e));
  return OR3_OK;
}

}  // namespace

extern "C" {

int or3_encode_rgb8(or3_context *ctx, const double *rgb, size_t n, int32_t gamma, uint8_t *out) {
  if (!ctx || (n && (!rgb || !out))) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  if (n == 0) return OR3_OK;
  cudaSetDevice(ctx->device);
  if (int e = ensure_gamma_table(ctx->device))
    return fail(ctx, OR3_ERR_CUDA, "gamma table: %s", cudaGetErrorString((cudaError_t)e));
  return transcode(ctx, rgb, 3 * n, out, 3 * n, [&](const double *i, uint8_t *o, cudaStream_t st) {
    launch_encode_rgb8(i, 3 * n, gamma ? 1 : 0, o, st);
  });
}

int or3_encode_rgbe(or3_context *ctx, const double *rgb, size_t n, uint8_t *out) {
  if (!ctx || (n && (!rgb || !out))) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  if (n == 0) return OR3_OK;
  cudaSetDevice(ctx->device);
  return transcode(ctx, rgb, 3 * n, out, 4 * n,
                   [&](const double *i, uint8_t *o, cudaStream_t st) { launch_encode_rgbe(i, n, o, st); });
}

int or3_decode_rgbe(or3_context *ctx, const uint8_t *rgbe, size_t n, float *out) {
  if (!ctx || (n && (!rgbe || !out))) return fail(ctx, OR3_ERR_INVALID_ARGUMENT, "null argument");
  if (n == 0) return OR3_OK;
  cudaSetDevice(ctx->device);
  return transcode(ctx, rgbe, 4 * n, out, 3 * n,
                   [&](const uint8_t *i, float *o, cudaStream_t st) { launch_decode_rgbe(i, n, o, st); });
}

int or3_get_frame_rgb8(or3_context *ctx, int32_t gamma, uint8_t *rgb, size_t capacity, int32_t *samples) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  if (int e = ensure_gamma_table(ctx->device))
    return fail(ctx, OR3_ERR_CUDA, "gamma table: %s", cudaGetErrorString((cudaError_t)e));
  return frame_bytes(ctx, rgb, capacity, samples, 3, [&](const double *f, size_t npix, uint8_t *o, cudaStream_t st) {
    launch_encode_rgb8(f, 3 * npix, gamma ? 1 : 0, o, st);
  });
}

int or3_get_frame_rgbe(or3_context *ctx, uint8_t *rgbe, size_t capacity, int32_t *samples) {
  if (!ctx) return OR3_ERR_INVALID_ARGUMENT;
  return frame_bytes(ctx, rgbe, capacity, samples, 4, [&](const double *f, size_t npix, uint8_t *o, cudaStream_t st) {
    launch_encode_rgbe(f, npix, o, st);
  });
}

}  // extern "C"
