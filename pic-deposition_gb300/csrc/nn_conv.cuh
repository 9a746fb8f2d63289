// 3x3 periodic convolutions on the tensor cores (tcgen05, BF16 in, FP32 accumulate).
//
// Tensors are NHWC BF16 with C in {16, 32}; W a multiple of 128 (forward and
// input-gradient kernels) and of 32 (weight-gradient kernel). Weights in
// "math" layout are FP32 w[tap][cout][cin], tap = (dy+1)*3 + (dx+1), and the
// forward convolution is
//     y[b,y,x,co] = bias[co] + sum_{dy,dx,ci} x[b,(y+dy)%H,(x+dx)%W,ci] * w[tap][co][ci].
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace picnn {

enum ConvEpilogue : int {
    EPI_BIAS_RELU = 0,  // y = relu(acc + bias), BF16 NHWC
    EPI_BIAS_OUT = 1,   // y = acc[channel 0] + bias[0], FP32, one value per pixel
    EPI_MASK = 2,       // y = acc * (mask > 0), BF16 NHWC (ReLU derivative of the layer below)
};

struct ConvLaunch {
    const uint16_t* x;     // input activations (BF16 bits), NHWC, cin channels
    const uint16_t* wimg;  // weight image: the B operand as it sits in shared memory
    const float* bias;     // cout values (EPI_BIAS_*)
    const uint16_t* mask;  // NHWC, cout channels (EPI_MASK)
    void* y;               // output
    int batch, H, W;
    int rows_per_cta;
    int* err;              // set to 1 when a wait on the tensor cores times out
};

struct WgradLaunch {
    const uint16_t* x;   // layer input, NHWC cin channels
    const uint16_t* dy;  // gradient at the layer output, NHWC cout channels
    float* partials;     // [grid][mpad][cout]
    int batch, H, W;
    int units_per_cta;   // blocks (8 rows x 32 pixels of one image) per CTA
    int* err;
    CUtensorMap tmx, tmdy;  // TMA views of x and dy (filled by launch_wgrad)
};

// Bytes of a weight image for (cin, cout).
inline size_t wimg_bytes(int cin, int cout) { return (size_t)9 * cin * cout * 2; }
// Rows of a weight-gradient partial sum: 9*cin taps-by-channels, then the bias.
inline int wgrad_mpad(int cin) { return 9 * cin + 1; }
// Blocks of the weight-gradient kernel: 8 rows x 32 pixels of one image.
inline long long wgrad_units(int batch, int H, int W) { return (long long)batch * ((H + 7) / 8) * (W / 32); }

// Forward convolution (transpose = 0) or the input gradient of layer (cin, cout)
// (transpose = 1: w'[tap][ci][co] = w[8 - tap][co][ci]) as a weight image.
int build_weight_image(const float* w_math, int cin, int cout, int transpose, uint16_t* img, cudaStream_t s);
// Launches one convolution; kcin/kcout are the kernel's channel counts.
int launch_conv(const ConvLaunch& a, int kcin, int kcout, int epilogue, cudaStream_t s);
// Weight gradient: partial sums per CTA (grid CTAs), then reduce_wgrad.
int launch_wgrad(const WgradLaunch& a, int cin, int cout, int grid, cudaStream_t s);
// dw[tap][co][ci] and db[co] from the partial sums of `grid` CTAs (fixed order).
int reduce_wgrad(const float* partials, int grid, int cin, int cout, float* dw, float* db, cudaStream_t s);
// CTAs the weight-gradient kernel uses for a problem of `units` blocks.
int wgrad_grid(long long units);

}  // namespace picnn
