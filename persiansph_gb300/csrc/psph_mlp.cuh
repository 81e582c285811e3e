// Learned eddy-viscosity closure: the network image the tensor-core kernels
// read, and the pieces the host API shares between psph_mlp.cu and psph_api.cu.
#pragma once

#include <stdint.h>

#include "psph.h"

namespace psph {

constexpr int kMlpIn = PSPH_MLP_INPUTS;   // 6 features
constexpr int kMlpH = PSPH_MLP_HIDDEN;    // 64 hidden units
constexpr int kMlpTile = 128;             // particles per tensor-core tile (MMA M)

// Offsets of the flattened FP32 parameters (include/psph.h order).
constexpr int kOW1 = 0;
constexpr int kOB1 = kOW1 + kMlpH * kMlpIn;   // 384
constexpr int kOW2 = kOB1 + kMlpH;            // 448
constexpr int kOB2 = kOW2 + kMlpH * kMlpH;    // 4544
constexpr int kOW3 = kOB2 + kMlpH;            // 4608
constexpr int kOB3 = kOW3 + kMlpH * kMlpH;    // 8704
constexpr int kOW4 = kOB3 + kMlpH;            // 8768
constexpr int kOB4 = kOW4 + kMlpH;            // 8832
constexpr int kNParams = kOB4 + 1;            // 8833
static_assert(kNParams == PSPH_MLP_NPARAMS, "parameter count");

// Operand images in shared-memory order: 64 rows (output units) x 64 BF16
// columns (input units, K-major), 128-byte swizzle: element (r, k) at byte
// (r/8)*1024 + (r%8)*128 + (((k/8) ^ (r%8)) * 16) + (k%8)*2. Layer 1 uses
// columns 0..15 (6 features, zero padded).
constexpr int kImgBytes = kMlpH * kMlpH * 2;  // 8192

struct MlpImage {
  uint8_t w1[kImgBytes];
  uint8_t w2[kImgBytes];
  uint8_t w3[kImgBytes];
  float b1[kMlpH], b2[kMlpH], b3[kMlpH], w4[kMlpH];
  float b4, pad0, pad1, pad2;
  float mean[kMlpIn], inv_std[kMlpIn], lo[kMlpIn], hi[kMlpIn];
};

// Byte offset of element (r, k) in a 128-byte-swizzled K-major operand.
inline __host__ __device__ int sw128_offset(int r, int k) {
  return (r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 3) ^ (r & 7)) & 7) << 4) + (k & 7) * 2;
}

}  // namespace psph

// Device image of a network (for psph_closure_attach).
psph_status psph_mlp_image(const psph_mlp* mlp, const psph::MlpImage** dev_image);
