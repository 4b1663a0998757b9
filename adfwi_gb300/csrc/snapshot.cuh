// Checkpoint snapshots of whole wavefield planes for the gradient's recomputation.
//
// A snapshot stores `nplanes` pitched planes (every field of every shot at one time step),
// either verbatim or as 16-bit values with one float max-abs scale per plane:
//   FP16: q = half(x / maxabs * 2^15)  (2^15 keeps |q| below the fp16 maximum of 65504 and
//         leaves values down to ~2e-9 of the plane's peak in the normal range);
//   BF16: q = bf16(x / maxabs);
// or as 24-bit floats without a scale:
//   FP24: the float32 value rounded to nearest (ties to even) at 15 mantissa bits, stored as its
//         upper 16 bits (a bfloat16 plane) and the next 8 bits (a byte plane): the float32
//         exponent range with a relative spacing of 2^-15, three bytes per value.
// The stencil arithmetic itself always stays in the wavefield type.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/adfwi_gb300.h"
#include "common.cuh"

namespace adfwi {

constexpr int kSnapThreads = 512;

template <typename T>
__device__ __forceinline__ float block_maxabs(const T* __restrict__ x, int64_t n) {
  __shared__ float red[kSnapThreads / 32];
  float m = 0.f;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) m = fmaxf(m, fabsf((float)x[e]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) red[0] = m;
  }
  __syncthreads();
  float r = red[0];
  __syncthreads();
  return r;
}

// One block per plane (blockIdx.x selects the plane; its threads stride the elements).
template <typename T, bool kHalf>
__global__ void __launch_bounds__(kSnapThreads) snap_quantize(const T* __restrict__ src, int64_t plane,
                                                              unsigned short* __restrict__ dst,
                                                              float* __restrict__ scales) {
  const int64_t pi = blockIdx.x;
  const T* x = src + pi * plane;
  const float m = block_maxabs(x, plane);
  if (threadIdx.x == 0) scales[pi] = m;
  const float inv = m > 0.f ? (kHalf ? 32768.f : 1.f) / m : 0.f;
  unsigned short* q = dst + pi * plane;
  for (int64_t e = threadIdx.x; e < plane; e += blockDim.x) {
    float v = (float)x[e] * inv;
    if (kHalf) {
      __half h = __float2half_rn(v);
      q[e] = *reinterpret_cast<unsigned short*>(&h);
    } else {
      __nv_bfloat16 b = __float2bfloat16_rn(v);
      q[e] = *reinterpret_cast<unsigned short*>(&b);
    }
  }
}

template <typename T, bool kHalf>
__global__ void __launch_bounds__(kSnapThreads) snap_dequantize(const unsigned short* __restrict__ src,
                                                                const float* __restrict__ scales, int64_t plane,
                                                                T* __restrict__ dst) {
  const int64_t pi = blockIdx.x;
  const float m = scales[pi];
  const float s = kHalf ? m / 32768.f : m;
  const unsigned short* q = src + pi * plane;
  T* y = dst + pi * plane;
  for (int64_t e = threadIdx.x; e < plane; e += blockDim.x) {
    unsigned short bits = q[e];
    float v;
    if (kHalf) {
      __half h = *reinterpret_cast<__half*>(&bits);
      v = __half2float(h);
    } else {
      __nv_bfloat16 b = *reinterpret_cast<__nv_bfloat16*>(&bits);
      v = __bfloat162float(b);
    }
    y[e] = (T)(v * s);
  }
}

// FP24: snapshot plane pi occupies bytes [3 pi plane, 3 (pi + 1) plane) of the store, its
// 16-bit upper parts first, then its 8-bit lower parts.
__device__ __forceinline__ unsigned fp24_round(float v) {
  const unsigned b = __float_as_uint(v);
  if ((b & 0x7f800000u) == 0x7f800000u) return b & 0xffffff00u;  // inf / nan: truncate
  return (b + 0x7fu + ((b >> 8) & 1u)) & 0xffffff00u;         // nearest, ties to even
}

template <typename T>
__global__ void snap_q24(const T* __restrict__ src, int64_t nplanes, int64_t plane, unsigned char* __restrict__ dst) {
  const int64_t n = nplanes * plane;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pi = e / plane, k = e - pi * plane;
    const unsigned r = fp24_round((float)src[e]);
    unsigned char* base = dst + pi * 3 * plane;
    reinterpret_cast<unsigned short*>(base)[k] = (unsigned short)(r >> 16);
    base[2 * plane + k] = (unsigned char)((r >> 8) & 0xffu);
  }
}

template <typename T>
__global__ void snap_dq24(const unsigned char* __restrict__ src, int64_t nplanes, int64_t plane, T* __restrict__ dst) {
  const int64_t n = nplanes * plane;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pi = e / plane, k = e - pi * plane;
    const unsigned char* base = src + pi * 3 * plane;
    const unsigned r = ((unsigned)reinterpret_cast<const unsigned short*>(base)[k] << 16) |
                       ((unsigned)base[2 * plane + k] << 8);
    dst[e] = (T)__uint_as_float(r);
  }
}

inline unsigned snap_blocks(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)(b < 152 * 32 ? (b < 1 ? 1 : b) : 152 * 32);
}

// Bytes per snapshot value of a precision (scales aside).
inline int snapshot_value_bytes(int prec, int elem) {
  return prec == ADFWI_SNAP_NATIVE ? elem : (prec == ADFWI_SNAP_FP24 ? 3 : 2);
}

// Store planes [0, nplanes) of `src` as snapshot planes [first, first + nplanes).
template <typename T>
int snapshot_store(int prec, const T* src, int64_t nplanes, int64_t plane, unsigned char* snap,
                   unsigned char* scales, int64_t first, cudaStream_t st) {
  if (prec == ADFWI_SNAP_NATIVE) {
    ADFWI_CUDA_TRY(cudaMemcpyAsync(snap + first * plane * (int64_t)sizeof(T), src, nplanes * plane * sizeof(T),
                                   cudaMemcpyDeviceToDevice, st));
    return kOk;
  }
  if (prec == ADFWI_SNAP_FP24) {
    ADFWI_LAUNCH(kAux, st, (snap_q24<T><<<snap_blocks(nplanes * plane), 256, 0, st>>>(src, nplanes, plane,
                                                                                    snap + first * 3 * plane)));
    ADFWI_CUDA_TRY(cudaGetLastError());
    return kOk;
  }
  unsigned short* q = reinterpret_cast<unsigned short*>(snap) + first * plane;
  float* sc = reinterpret_cast<float*>(scales) + first;
  if (prec == ADFWI_SNAP_FP16)
    ADFWI_LAUNCH(kAux, st, (snap_quantize<T, true><<<(unsigned)nplanes, kSnapThreads, 0, st>>>(src, plane, q, sc)));
  else
    ADFWI_LAUNCH(kAux, st, (snap_quantize<T, false><<<(unsigned)nplanes, kSnapThreads, 0, st>>>(src, plane, q, sc)));
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

template <typename T>
int snapshot_load(int prec, T* dst, int64_t nplanes, int64_t plane, const unsigned char* snap,
                  const unsigned char* scales, int64_t first, cudaStream_t st) {
  if (prec == ADFWI_SNAP_NATIVE) {
    ADFWI_CUDA_TRY(cudaMemcpyAsync(dst, snap + first * plane * (int64_t)sizeof(T), nplanes * plane * sizeof(T),
                                   cudaMemcpyDeviceToDevice, st));
    return kOk;
  }
  if (prec == ADFWI_SNAP_FP24) {
    ADFWI_LAUNCH(kAux, st, (snap_dq24<T><<<snap_blocks(nplanes * plane), 256, 0, st>>>(snap + first * 3 * plane,
                                                                                     nplanes, plane, dst)));
    ADFWI_CUDA_TRY(cudaGetLastError());
    return kOk;
  }
  const unsigned short* q = reinterpret_cast<const unsigned short*>(snap) + first * plane;
  const float* sc = reinterpret_cast<const float*>(scales) + first;
  if (prec == ADFWI_SNAP_FP16)
    ADFWI_LAUNCH(kAux, st, (snap_dequantize<T, true><<<(unsigned)nplanes, kSnapThreads, 0, st>>>(q, sc, plane, dst)));
  else
    ADFWI_LAUNCH(kAux, st, (snap_dequantize<T, false><<<(unsigned)nplanes, kSnapThreads, 0, st>>>(q, sc, plane, dst)));
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace adfwi
