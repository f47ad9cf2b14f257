// pt_detector.cu -- detector acceptance of particle rows on the device:
// PETITE's detector_cut (shower.py:825-865) with its transverse_position
// (shower.py:815-823), over SoA rows already in HBM (a pt_particles store's
// p0/r0, or the dark vectors of pt_dark_out).  sm_103a only.
//
// Per row and disk detector at longitudinal position z: the initial straight
// line reaches z at T = (z - z0)/pz, (x, y) = (x0 + T px, y0 + T py), and the
// row passes when r_inner < sqrt(x^2 + y^2) < r_outer, after the optional
// open energy window e_min < E < e_max.  Every operation is rounded on its
// own (no fused multiply-add), as numpy evaluates the reference's array
// expressions, so the pass mask is bit-for-bit the reference's.
//
// The kernel streams each row's eight doubles (E, px, py, pz, x0, y0, z0,
// weight) once per group of up to kGroup detectors: 64 B per row read, one
// byte per row and detector written.  It screens rows in float32 (the
// float64 pipe is 1/63 of the float32 rate on this GPU) and recomputes in
// float64 only the rows the screen cannot decide.  The grid is sized to the
// rows, capped at the resident blocks with grid-stride loops.
#include <cstdint>
#include <cuda_runtime.h>

#include "petite_gpu.h"

namespace {

constexpr int kGroup = 4;           // detectors per pass over the rows
constexpr int kThreads = 256;

// float32 of a double from its high word alone, by integer operations:
// sign, exponent rebased, the top 20 mantissa bits (truncated, relative
// error below 2^-20).  Magnitudes below 2^-126 give 0; above float32's range,
// infinities and NaNs give infinity.  (A float64-to-float32 conversion
// instruction runs on the narrow float64 pipe.)
__device__ __forceinline__ float f32_hi(double d) {
  const unsigned hi = (unsigned)__double2hiint(d);
  const int e = (int)((hi >> 20) & 0x7FFu) - 896;      // 1023 - 127
  const unsigned sgn = hi & 0x80000000u;
  const unsigned bits = e <= 0 ? sgn : (e >= 255 ? (sgn | 0x7F800000u) : (sgn | ((unsigned)e << 23) | ((hi & 0xFFFFFu) << 3)));
  return __uint_as_float(bits);
}

// The reference's arithmetic for one row and detector, each operation
// rounded on its own: r_T = sqrt(x^2 + y^2) at T = (z - z0)/pz.
__device__ __forceinline__ bool pass_exact(double z, double x0, double y0, double z0, double px, double py, double pz,
                                           double r_inner, double r_outer) {
  const double T = __ddiv_rn(__dsub_rn(z, z0), pz);
  const double xf = __dadd_rn(x0, __dmul_rn(T, px)), yf = __dadd_rn(y0, __dmul_rn(T, py));
  const double rT = __dsqrt_rn(__dadd_rn(__dmul_rn(xf, xf), __dmul_rn(yf, yf)));
  return rT > r_inner && rT < r_outer;
}

// Each row is first screened in float32 from the inputs' high words.  With
// S = |x0| + |y0| + (|z| + |z0|)(|px| + |py|)/|pz|, the screen's r_T^2 is
// within 8 * 2^-20 S^2 of the exact one (inputs truncated to 2^-20,
// approximate division 2 ulp, float32 roundings); the margin M = 2^-16 S^2
// (twice that) plus 2^-19 of the threshold decides the row only when both
// annulus edges are clear of it.  Otherwise, whenever a value is not finite,
// and for |pz| beyond 2^126 (where the approximate division returns 0), the
// row takes the exact path.  The decisions are the exact ones.
__global__ void __launch_bounds__(kThreads, 4) k_detector_cut(const double* __restrict__ p4, int64_t p4_stride,
                                                           const double* __restrict__ r, int64_t r_stride,
                                                           const double* __restrict__ weight, int64_t n,
                                                           const double* __restrict__ z_det, int d0, int nd,
                                                           double r_inner, double r_outer, int use_window,
                                                           double e_min, double e_max, uint8_t* __restrict__ pass,
                                                           double* __restrict__ sums, int n_det, int count_total) {
  __shared__ double red[kThreads / 32][kGroup + 1];
  const float ro2 = f32_hi(r_outer * r_outer), ri2 = f32_hi(r_inner * r_inner);
  const float mo = 0x1p-19f * ro2, mi = 0x1p-19f * ri2;   // threshold truncation (2^-20) with room
  double acc[kGroup + 1];
#pragma unroll
  for (int k = 0; k <= kGroup; ++k) acc[k] = 0.0;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    const double px = __ldg(p4 + p4_stride + i), py = __ldg(p4 + 2 * p4_stride + i),
                 pz = __ldg(p4 + 3 * p4_stride + i);
    const double x0 = __ldg(r + i), y0 = __ldg(r + r_stride + i), z0 = __ldg(r + 2 * r_stride + i);
    bool in = true;
    if (use_window) {
      const double E = __ldg(p4 + i);
      in = E < e_max && E > e_min;
    }
    const double w = sums ? (weight ? __ldg(weight + i) : 1.0) : 0.0;
    if (in && sums) acc[kGroup] += w;
    const float pxf = f32_hi(px), pyf = f32_hi(py), pzf = f32_hi(pz);
    const float x0f = f32_hi(x0), y0f = f32_hi(y0), z0f = f32_hi(z0);
    const float ipz = __fdividef(1.f, fabsf(pzf));
    const float sxy = fabsf(pxf) + fabsf(pyf);
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {
      if (k >= nd) break;
      const double z = __ldg(z_det + d0 + k);
      const float zf = f32_hi(z);
      const float T = __fdividef(zf - z0f, pzf);
      const float xf = fmaf(T, pxf, x0f), yf = fmaf(T, pyf, y0f);
      const float s2 = fmaf(xf, xf, yf * yf);
      const float S = fabsf(x0f) + fabsf(y0f) + (fabsf(zf) + fabsf(z0f)) * sxy * ipz;
      const float M = 0x1p-16f * S * S + 1e-30f;
      const bool out_yes = s2 < ro2 - (M + mo), out_no = s2 > ro2 + (M + mo);
      const bool in_yes = s2 > ri2 + (M + mi), in_no = s2 < ri2 - (M + mi);
      bool ok;
      if (fabsf(pzf) < 0x1p126f && (out_yes || out_no) && (in_yes || in_no)) ok = out_yes && in_yes;
      else ok = pass_exact(z, x0, y0, z0, px, py, pz, r_inner, r_outer);
      ok = ok && in;
      if (pass) pass[(int64_t)(d0 + k) * n + i] = ok ? 1 : 0;
      if (ok && sums) acc[k] += w;
    }
  }
  if (!sums) return;
  // block sums: warp shuffles, then the block's warps in order; one atomic
  // add per detector per block
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k <= kGroup; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x <= kGroup) {
    const int k = threadIdx.x;
    double v = 0.0;
    for (int j = 0; j < kThreads / 32; ++j) v += red[j][k];
    if (k < nd && v != 0.0) atomicAdd(sums + d0 + k, v);
    if (k == kGroup && count_total && v != 0.0) atomicAdd(sums + n_det, v);
  }
}

}  // namespace

extern "C" pt_status pt_detector_cut(const double* p4, int64_t p4_stride, const double* r, int64_t r_stride,
                                     const double* weight, int64_t n, const double* z_det, int32_t n_det,
                                     double r_inner, double r_outer, int32_t use_window, double e_min, double e_max,
                                     uint8_t* pass, double* sums, void* stream) {
  if (n < 0 || n_det < 0 || (n > 0 && (!p4 || !r || p4_stride < n || r_stride < n)) || (n_det > 0 && !z_det))
    return PT_BAD_ARG;
  const cudaStream_t st = (cudaStream_t)stream;
  if (sums && cudaMemsetAsync(sums, 0, (size_t)(n_det + 1) * sizeof(double), st) != cudaSuccess) return PT_CUDA_ERR;
  if (n == 0 || (n_det == 0 && !sums)) return cudaGetLastError() == cudaSuccess ? PT_OK : PT_CUDA_ERR;
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_detector_cut, kThreads, 0);
  if (sms < 1) sms = 1;
  if (per < 1) per = 1;
  const int64_t want = (n + kThreads - 1) / kThreads, cap = (int64_t)sms * per;   // the resident blocks
  const int blocks = (int)(want < cap ? want : cap);
  // one pass over the rows per group of detectors; the first pass also
  // sums the window's total weight (a pass with no detector when n_det = 0)
  for (int d0 = 0; d0 < n_det || d0 == 0; d0 += kGroup) {
    const int nd = n_det - d0 < kGroup ? n_det - d0 : kGroup;
    k_detector_cut<<<blocks, kThreads, 0, st>>>(p4, p4_stride, r, r_stride, weight, n, z_det, d0, nd > 0 ? nd : 0,
                                                r_inner, r_outer, use_window, e_min, e_max, pass, sums, n_det,
                                                d0 == 0 ? 1 : 0);
    if (cudaGetLastError() != cudaSuccess) return PT_CUDA_ERR;
    if (n_det == 0) break;
  }
  return PT_OK;
}
