// Device scratch of the GPU SAH batching (sah_gpu.cu): n elements each unless
// noted, carved from one buffer by the caller (capi.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace occ {

struct SahScratch {
  float4* lo;                  // box minima
  float4* hi;                  // box maxima
  uint32_t* mk;                // 3 x n: centre keys per axis (order-preserving, the two zeros alike)
  uint32_t* idx[2];            // quad order (ping-pong)
  unsigned long long* key[2];  // sort keys (ping-pong)
  uint32_t* rng;               // range of each position
  float* left;                 // surface area of the range's prefix union ending at each position
  float* right;                // ... of the suffix union starting at each position
  uint32_t* hist;              // 256 x sort tiles
  uint32_t* starts;            // range starts + n (capacity n + 1)
  int8_t* rangeAxis;           // per range: axis whose centre keys it sorts by, -1: none (capacity n)
  unsigned long long* best;    // per range: cheapest split (capacity n)
  float4* aggLo;               // per scan tile: segmented aggregate (box, starts-a-range flag in .w)
  float4* aggHi;
  uint32_t* flag;              // [0]: a NaN centre was seen
};

}  // namespace occ
