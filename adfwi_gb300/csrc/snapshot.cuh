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

// Each plane is split into chunks of kSnapChunk elements, one block per (chunk, plane): the
// max-abs pass combines the chunks' maxima by atomicMax on the bit patterns of the non-negative
// floats (exact and order-independent: the scale is the plane's max |x| whatever the split),
// then the (de)quantising passes run over the same grid.
constexpr int kSnapChunk = 8192;

inline dim3 snap_grid(int64_t nplanes, int64_t plane) {
  return dim3((unsigned)((plane + kSnapChunk - 1) / kSnapChunk), (unsigned)nplanes);
}

template <typename T>
__global__ void __launch_bounds__(kSnapThreads) snap_maxabs(const T* __restrict__ src, int64_t plane,
                                                            unsigned* __restrict__ scale_bits) {
  __shared__ float red[kSnapThreads / 32];
  const int64_t pi = blockIdx.y, b0 = (int64_t)blockIdx.x * kSnapChunk;
  const int64_t b1 = b0 + kSnapChunk < plane ? b0 + kSnapChunk : plane;
  const T* x = src + pi * plane;
  float m = 0.f;
  for (int64_t e = b0 + threadIdx.x; e < b1; e += blockDim.x) m = fmaxf(m, fabsf((float)x[e]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) atomicMax(scale_bits + pi, __float_as_uint(m));
  }
}

template <typename T, bool kHalf>
__global__ void __launch_bounds__(kSnapThreads) snap_quantize(const T* __restrict__ src, int64_t plane,
                                                              unsigned short* __restrict__ dst,
                                                              const float* __restrict__ scales) {
  const int64_t pi = blockIdx.y, b0 = (int64_t)blockIdx.x * kSnapChunk;
  const int64_t b1 = b0 + kSnapChunk < plane ? b0 + kSnapChunk : plane;
  const T* x = src + pi * plane;
  const float m = scales[pi];
  const float inv = m > 0.f ? (kHalf ? 32768.f : 1.f) / m : 0.f;
  unsigned short* q = dst + pi * plane;
  for (int64_t e = b0 + threadIdx.x; e < b1; e += blockDim.x) {
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
  const int64_t pi = blockIdx.y, b0 = (int64_t)blockIdx.x * kSnapChunk;
  const int64_t b1 = b0 + kSnapChunk < plane ? b0 + kSnapChunk : plane;
  const float m = scales[pi];
  const float s = kHalf ? m / 32768.f : m;
  const unsigned short* q = src + pi * plane;
  T* y = dst + pi * plane;
  for (int64_t e = b0 + threadIdx.x; e < b1; e += blockDim.x) {
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
__global__ void __launch_bounds__(kSnapThreads) snap_q24(const T* __restrict__ src, int64_t plane,
                                                         unsigned char* __restrict__ dst) {
  const int64_t pi = blockIdx.y, b0 = (int64_t)blockIdx.x * kSnapChunk;
  const int64_t b1 = b0 + kSnapChunk < plane ? b0 + kSnapChunk : plane;
  const T* x = src + pi * plane;
  unsigned char* base = dst + pi * 3 * plane;
  for (int64_t k = b0 + threadIdx.x; k < b1; k += blockDim.x) {
    const unsigned r = fp24_round((float)x[k]);
    reinterpret_cast<unsigned short*>(base)[k] = (unsigned short)(r >> 16);
    base[2 * plane + k] = (unsigned char)((r >> 8) & 0xffu);
  }
}

template <typename T>
__global__ void __launch_bounds__(kSnapThreads) snap_dq24(const unsigned char* __restrict__ src, int64_t plane,
                                                          T* __restrict__ dst) {
  const int64_t pi = blockIdx.y, b0 = (int64_t)blockIdx.x * kSnapChunk;
  const int64_t b1 = b0 + kSnapChunk < plane ? b0 + kSnapChunk : plane;
  const unsigned char* base = src + pi * 3 * plane;
  T* y = dst + pi * plane;
  for (int64_t k = b0 + threadIdx.x; k < b1; k += blockDim.x) {
    const unsigned r = ((unsigned)reinterpret_cast<const unsigned short*>(base)[k] << 16) |
                       ((unsigned)base[2 * plane + k] << 8);
    y[k] = (T)__uint_as_float(r);
  }
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
  if (nplanes > 65535) {
    set_error("snapshot of %lld planes: at most 65535 per store", (long long)nplanes);
    return kBadArgument;
  }
  if (prec == ADFWI_SNAP_FP24) {
    ADFWI_LAUNCH(kAux, st, (snap_q24<T><<<snap_grid(nplanes, plane), kSnapThreads, 0, st>>>(
                               src, plane, snap + first * 3 * plane)));
    ADFWI_CUDA_TRY(cudaGetLastError());
    return kOk;
  }
  unsigned short* q = reinterpret_cast<unsigned short*>(snap) + first * plane;
  float* sc = reinterpret_cast<float*>(scales) + first;
  const dim3 grid = snap_grid(nplanes, plane);
  ADFWI_CUDA_TRY(cudaMemsetAsync(sc, 0, nplanes * sizeof(float), st));  // maxima start at +0
  ADFWI_LAUNCH(kAux, st, (snap_maxabs<T><<<grid, kSnapThreads, 0, st>>>(src, plane, reinterpret_cast<unsigned*>(sc))));
  if (prec == ADFWI_SNAP_FP16)
    ADFWI_LAUNCH(kAux, st, (snap_quantize<T, true><<<grid, kSnapThreads, 0, st>>>(src, plane, q, sc)));
  else
    ADFWI_LAUNCH(kAux, st, (snap_quantize<T, false><<<grid, kSnapThreads, 0, st>>>(src, plane, q, sc)));
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
  if (nplanes > 65535) {
    set_error("snapshot of %lld planes: at most 65535 per load", (long long)nplanes);
    return kBadArgument;
  }
  if (prec == ADFWI_SNAP_FP24) {
    ADFWI_LAUNCH(kAux, st, (snap_dq24<T><<<snap_grid(nplanes, plane), kSnapThreads, 0, st>>>(
                               snap + first * 3 * plane, plane, dst)));
    ADFWI_CUDA_TRY(cudaGetLastError());
    return kOk;
  }
  const unsigned short* q = reinterpret_cast<const unsigned short*>(snap) + first * plane;
  const float* sc = reinterpret_cast<const float*>(scales) + first;
  const dim3 grid = snap_grid(nplanes, plane);
  if (prec == ADFWI_SNAP_FP16)
    ADFWI_LAUNCH(kAux, st, (snap_dequantize<T, true><<<grid, kSnapThreads, 0, st>>>(q, sc, plane, dst)));
  else
    ADFWI_LAUNCH(kAux, st, (snap_dequantize<T, false><<<grid, kSnapThreads, 0, st>>>(q, sc, plane, dst)));
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace adfwi
