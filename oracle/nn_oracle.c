/* CPU oracle of the learned warm start's convolution network -- TEST INFRASTRUCTURE ONLY.
 *
 * No reference code exists for this part (the reference has no network); these
 * are plain restatements of the definitions the GPU kernels implement:
 *   3x3 periodic convolution, NHWC tensors, weights w[tap][cout][cin] with
 *   tap = (dy+1)*3 + (dx+1):  y[p][co] = b[co] + sum_{tap,ci} x[p+tap][ci] w[tap][co][ci]
 * and its two gradients (input: the transposed convolution with flipped taps;
 * weights: the correlation of the layer input with the output gradient).
 * Sums are FP64. BF16 values are the upper 16 bits of an IEEE binary32, rounded
 * to nearest even -- the same points at which the GPU path rounds (weights,
 * stored activations, stored gradients) are rounded here when `quantize` is set.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static float bf16_to_f(uint16_t h) {
    uint32_t u = (uint32_t)h << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

static uint16_t f_to_bf16(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u && (u & 0x007FFFFFu)) return (uint16_t)((u >> 16) | 0x40u); /* NaN */
    const uint32_t lsb = (u >> 16) & 1u;
    u += 0x7FFFu + lsb;
    return (uint16_t)(u >> 16);
}

uint16_t orc_bf16_from_float(float f) { return f_to_bf16(f); }
float orc_float_from_bf16(uint16_t h) { return bf16_to_f(h); }

static double q(double v, int quantize) { return quantize ? (double)bf16_to_f(f_to_bf16((float)v)) : v; }

static size_t pix(int b, int y, int x, int H, int W) {
    return ((size_t)b * H + (size_t)((y % H + H) % H)) * W + (size_t)((x % W + W) % W);
}

/* acc[p][co] = sum_{tap,ci} x[p+tap][ci] * w[tap][co][ci]   (x, w as doubles) */
static void conv_fwd_d(int B, int H, int W, int cin, int cout, const double* x, const double* w, double* acc) {
    for (int b = 0; b < B; ++b)
        for (int y = 0; y < H; ++y)
            for (int xx = 0; xx < W; ++xx) {
                double* o = acc + pix(b, y, xx, H, W) * cout;
                for (int co = 0; co < cout; ++co) o[co] = 0.0;
                for (int t = 0; t < 9; ++t) {
                    const double* in = x + pix(b, y + t / 3 - 1, xx + t % 3 - 1, H, W) * cin;
                    for (int co = 0; co < cout; ++co) {
                        const double* wr = w + ((size_t)t * cout + co) * cin;
                        double s = 0.0;
                        for (int ci = 0; ci < cin; ++ci) s += in[ci] * wr[ci];
                        o[co] += s;
                    }
                }
            }
}

/* acc[p][ci] = sum_{tap,co} dy[p-tap][co] * w[tap][co][ci] */
static void conv_dgrad_d(int B, int H, int W, int cin, int cout, const double* dy, const double* w, double* acc) {
    for (int b = 0; b < B; ++b)
        for (int y = 0; y < H; ++y)
            for (int xx = 0; xx < W; ++xx) {
                double* o = acc + pix(b, y, xx, H, W) * cin;
                for (int ci = 0; ci < cin; ++ci) o[ci] = 0.0;
                for (int t = 0; t < 9; ++t) {
                    const double* g = dy + pix(b, y - (t / 3 - 1), xx - (t % 3 - 1), H, W) * cout;
                    for (int co = 0; co < cout; ++co) {
                        const double* wr = w + ((size_t)t * cout + co) * cin;
                        for (int ci = 0; ci < cin; ++ci) o[ci] += g[co] * wr[ci];
                    }
                }
            }
}

/* dw[tap][co][ci] = sum_p x[p+tap][ci] dy[p][co]; db[co] = sum_p dy[p][co] */
static void conv_wgrad_d(int B, int H, int W, int cin, int cout, const double* x, const double* dy, double* dw,
                         double* db) {
    memset(dw, 0, sizeof(double) * 9 * cin * cout);
    memset(db, 0, sizeof(double) * cout);
    for (int b = 0; b < B; ++b)
        for (int y = 0; y < H; ++y)
            for (int xx = 0; xx < W; ++xx) {
                const double* g = dy + pix(b, y, xx, H, W) * cout;
                for (int co = 0; co < cout; ++co) db[co] += g[co];
                for (int t = 0; t < 9; ++t) {
                    const double* in = x + pix(b, y + t / 3 - 1, xx + t % 3 - 1, H, W) * cin;
                    for (int co = 0; co < cout; ++co) {
                        double* d = dw + ((size_t)t * cout + co) * cin;
                        for (int ci = 0; ci < cin; ++ci) d[ci] += in[ci] * g[co];
                    }
                }
            }
}

static double* bf16_array(const uint16_t* h, size_t n) {
    double* d = (double*)malloc(sizeof(double) * (n ? n : 1));
    for (size_t i = 0; i < n; ++i) d[i] = bf16_to_f(h[i]);
    return d;
}

static double* weights_bf16(const float* w, size_t n) {
    double* d = (double*)malloc(sizeof(double) * n);
    for (size_t i = 0; i < n; ++i) d[i] = bf16_to_f(f_to_bf16(w[i]));
    return d;
}

/* epi 0: out bf16 relu(acc + bias), cout channels; epi 1: out FP32 acc[0] + bias[0] */
int orc_conv3x3_fwd(int B, int H, int W, int cin, int cout, const uint16_t* x, const float* w, const float* bias,
                    int epi, void* out) {
    const size_t P = (size_t)B * H * W;
    double* xd = bf16_array(x, P * cin);
    double* wd = weights_bf16(w, (size_t)9 * cin * cout);
    double* acc = (double*)malloc(sizeof(double) * P * cout);
    conv_fwd_d(B, H, W, cin, cout, xd, wd, acc);
    for (size_t p = 0; p < P; ++p) {
        if (epi == 1) {
            ((float*)out)[p] = (float)acc[p * cout] + bias[0];
        } else {
            for (int c = 0; c < cout; ++c) {
                float v = (float)acc[p * cout + c] + bias[c];
                ((uint16_t*)out)[p * cout + c] = f_to_bf16(v > 0.0f ? v : 0.0f);
            }
        }
    }
    free(xd);
    free(wd);
    free(acc);
    return 0;
}

int orc_conv3x3_dgrad(int B, int H, int W, int cin, int cout, const uint16_t* dy, const float* w, const uint16_t* mask,
                      uint16_t* dx) {
    const size_t P = (size_t)B * H * W;
    double* gd = bf16_array(dy, P * cout);
    double* wd = weights_bf16(w, (size_t)9 * cin * cout);
    double* acc = (double*)malloc(sizeof(double) * P * cin);
    conv_dgrad_d(B, H, W, cin, cout, gd, wd, acc);
    for (size_t i = 0; i < P * cin; ++i) {
        const int16_t m = (int16_t)mask[i];
        dx[i] = f_to_bf16(m > 0 ? (float)acc[i] : 0.0f);
    }
    free(gd);
    free(wd);
    free(acc);
    return 0;
}

int orc_conv3x3_wgrad(int B, int H, int W, int cin, int cout, const uint16_t* x, const uint16_t* dy, double* dw,
                      double* db) {
    const size_t P = (size_t)B * H * W;
    double* xd = bf16_array(x, P * cin);
    double* gd = bf16_array(dy, P * cout);
    conv_wgrad_d(B, H, W, cin, cout, xd, gd, dw, db);
    free(xd);
    free(gd);
    return 0;
}

/* ---- the warm-start network: 6 layers, channels 16(1 used)->32->32->32->32->32->16(1 used) ---- */
#define NN_LAYERS 6
static const int NN_CIN[NN_LAYERS] = {16, 32, 32, 32, 32, 32};
static const int NN_COUT[NN_LAYERS] = {32, 32, 32, 32, 32, 16};

size_t orc_net_param_count(void) {
    size_t n = 0;
    for (int l = 0; l < NN_LAYERS; ++l) n += (size_t)9 * NN_CIN[l] * NN_COUT[l] + NN_COUT[l];
    return n;
}

/* Loss L = mean_p (out[p] - target[p])^2 with out = layer 6 channel 0, and dL/dparams
 * (same flat layout as params: per layer w[9][cout][cin] then b[cout]).
 * input: B*H*W values in channel 0 (channels 1..15 zero). With quantize set, the
 * weights, the input, every stored activation and every stored gradient are
 * rounded to BF16 at the points where the GPU path stores them. */
int orc_net_loss_grad(int B, int H, int W, const float* params, const float* input, const float* target, int quantize,
                      double* loss, double* grad) {
    const size_t P = (size_t)B * H * W;
    double* a[NN_LAYERS + 1];
    double* wl[NN_LAYERS];
    const float* bl[NN_LAYERS];
    size_t off = 0;
    for (int l = 0; l < NN_LAYERS; ++l) {
        const size_t nw = (size_t)9 * NN_CIN[l] * NN_COUT[l];
        wl[l] = (double*)malloc(sizeof(double) * nw);
        for (size_t i = 0; i < nw; ++i) wl[l][i] = q(params[off + i], quantize);
        bl[l] = params + off + nw;
        off += nw + NN_COUT[l];
    }
    a[0] = (double*)calloc(P * 16, sizeof(double));
    for (size_t p = 0; p < P; ++p) a[0][p * 16] = q(input[p], quantize);
    for (int l = 0; l < NN_LAYERS; ++l) {
        a[l + 1] = (double*)malloc(sizeof(double) * P * NN_COUT[l]);
        conv_fwd_d(B, H, W, NN_CIN[l], NN_COUT[l], a[l], wl[l], a[l + 1]);
        for (size_t p = 0; p < P; ++p)
            for (int c = 0; c < NN_COUT[l]; ++c) {
                double v = a[l + 1][p * NN_COUT[l] + c];
                if (quantize) v = (double)((float)v + bl[l][c]);
                else v += (double)bl[l][c];
                if (l < NN_LAYERS - 1) v = q(v > 0.0 ? v : 0.0, quantize);
                a[l + 1][p * NN_COUT[l] + c] = v;
            }
    }
    /* loss and its gradient at the output (channel 0 of 16) */
    double L = 0.0;
    double* g = (double*)calloc(P * 16, sizeof(double));
    for (size_t p = 0; p < P; ++p) {
        const double out = quantize ? (double)(float)a[NN_LAYERS][p * 16] : a[NN_LAYERS][p * 16];
        const double d = out - (double)target[p];
        L += d * d;
        g[p * 16] = q(2.0 * d / (double)P, quantize);
    }
    *loss = L / (double)P;
    size_t goff = off;
    for (int l = NN_LAYERS - 1; l >= 0; --l) {
        const int cin = NN_CIN[l], cout = NN_COUT[l];
        const size_t nw = (size_t)9 * cin * cout;
        goff -= nw + cout;
        conv_wgrad_d(B, H, W, cin, cout, a[l], g, grad + goff, grad + goff + nw);
        if (l > 0) {
            double* gin = (double*)malloc(sizeof(double) * P * cin);
            conv_dgrad_d(B, H, W, cin, cout, g, wl[l], gin);
            for (size_t i = 0; i < P * cin; ++i) gin[i] = a[l][i] > 0.0 ? q(gin[i], quantize) : 0.0;
            free(g);
            g = gin;
        }
    }
    free(g);
    for (int l = 0; l <= NN_LAYERS; ++l) free(a[l]);
    for (int l = 0; l < NN_LAYERS; ++l) free(wl[l]);
    return 0;
}
