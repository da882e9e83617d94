// Min-max pyramid of a light map (internal): level L in 1..6 holds
// float2(min, max) of every 2^L x 2^L texel block, row-major over
// (W >> L) x (H >> L) cells.  Built by launch_minmax_pyramid (minmax.cu),
// read by the visibility kernels to skip taps whose outcome it decides.
#pragma once

#include <cuda_runtime.h>

#include "internal.h"

namespace gi {

constexpr int kPyramidLevels = 6;

struct Pyramid {
    float2* lv[kPyramidLevels + 1];  // lv[0] unused (level 0 is the map)
    int levels;                      // 0: no pyramid
};

// Sides must be multiples of 64 (one CTA per 64 x 64 tile).
bool pyramid_supported(int W, int H);
// Builds the pyramid of d_map into the context's scratch; *out.levels is 0
// (and nothing is launched) when the map's shape is not supported.
gi_status launch_minmax_pyramid(gi_context* ctx, const float* d_map, int W, int H, cudaStream_t st, Pyramid* out);

}  // namespace gi
