/*
 * FFTW3-API shim (test infrastructure; see fftw3.h).
 *
 * A 1-D real transform of length n in FFTW's halfcomplex order is
 *   R2HC:  out[k] = Re X_k (0 <= k <= n/2),  out[n-k] = Im X_k (0 < k < (n+1)/2),
 *          X_k = sum_j x_j exp(-2 pi i j k / n)
 *   HC2R:  the unnormalised inverse, x_j = sum_k X_k exp(+2 pi i j k / n),
 *          with X_{n-k} = conj(X_k).
 * A 2-D r2r plan applies the 1-D kind of each dimension along that dimension
 * (row-major n0 x n1 array), which is what FFTW documents for r2r_2d.
 *
 * Each line is transformed with an iterative radix-2 complex FFT when n is a
 * power of two, and with a direct O(n^2) DFT otherwise.
 */
#include "fftw3.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct pic_shim_fftw_plan_s {
    int n0, n1;
    double* in;
    double* out;
    fftw_r2r_kind k0, k1;
};

double* fftw_alloc_real(size_t n) { return (double*)malloc((n ? n : 1) * sizeof(double)); }

void fftw_free(void* p) { free(p); }

fftw_plan fftw_plan_r2r_2d(int n0, int n1, double* in, double* out, fftw_r2r_kind kind0, fftw_r2r_kind kind1,
                           unsigned flags) {
    (void)flags;
    fftw_plan p = (fftw_plan)malloc(sizeof(*p));
    p->n0 = n0;
    p->n1 = n1;
    p->in = in;
    p->out = out;
    p->k0 = kind0;
    p->k1 = kind1;
    return p;
}

void fftw_destroy_plan(fftw_plan plan) { free(plan); }

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* In-place complex transform of (re, im), sign = -1 forward, +1 backward. */
static void cfft(double* re, double* im, int n, int sign) {
    if (n <= 1) return;
    if (is_pow2(n)) {
        for (int i = 1, j = 0; i < n; ++i) {
            int bit = n >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) {
                double t = re[i];
                re[i] = re[j];
                re[j] = t;
                t = im[i];
                im[i] = im[j];
                im[j] = t;
            }
        }
        for (int len = 2; len <= n; len <<= 1) {
            const int half = len >> 1;
            for (int k = 0; k < half; ++k) {
                const double ang = sign * 2.0 * M_PI * (double)k / (double)len;
                const double wr = cos(ang), wi = sin(ang);
                for (int s = 0; s < n; s += len) {
                    const int a = s + k, b = s + k + half;
                    const double xr = re[b] * wr - im[b] * wi;
                    const double xi = re[b] * wi + im[b] * wr;
                    re[b] = re[a] - xr;
                    im[b] = im[a] - xi;
                    re[a] += xr;
                    im[a] += xi;
                }
            }
        }
        return;
    }
    double* tr = (double*)malloc((size_t)n * sizeof(double));
    double* ti = (double*)malloc((size_t)n * sizeof(double));
    for (int k = 0; k < n; ++k) {
        double sr = 0.0, si = 0.0;
        for (int j = 0; j < n; ++j) {
            const double ang = sign * 2.0 * M_PI * (double)(((long long)j * k) % n) / (double)n;
            sr += re[j] * cos(ang) - im[j] * sin(ang);
            si += re[j] * sin(ang) + im[j] * cos(ang);
        }
        tr[k] = sr;
        ti[k] = si;
    }
    memcpy(re, tr, (size_t)n * sizeof(double));
    memcpy(im, ti, (size_t)n * sizeof(double));
    free(tr);
    free(ti);
}

/* One strided line: data[off + i*stride], i < n. */
static void line_r2r(double* data, int n, int stride, fftw_r2r_kind kind, double* re, double* im) {
    if (kind == FFTW_R2HC) {
        for (int i = 0; i < n; ++i) {
            re[i] = data[(size_t)i * stride];
            im[i] = 0.0;
        }
        cfft(re, im, n, -1);
        for (int k = 0; k <= n / 2; ++k) data[(size_t)k * stride] = re[k];
        for (int k = 1; k < (n + 1) / 2; ++k) data[(size_t)(n - k) * stride] = im[k];
    } else {
        re[0] = data[0];
        im[0] = 0.0;
        for (int k = 1; k < (n + 1) / 2; ++k) {
            const double r = data[(size_t)k * stride];
            const double i = data[(size_t)(n - k) * stride];
            re[k] = r;
            im[k] = i;
            re[n - k] = r;
            im[n - k] = -i;
        }
        if (n % 2 == 0) {
            re[n / 2] = data[(size_t)(n / 2) * stride];
            im[n / 2] = 0.0;
        }
        cfft(re, im, n, +1);
        for (int j = 0; j < n; ++j) data[(size_t)j * stride] = re[j];
    }
}

void fftw_execute(const fftw_plan p) {
    const int n0 = p->n0, n1 = p->n1;
    const size_t total = (size_t)n0 * (size_t)n1;
    if (p->out != p->in) memcpy(p->out, p->in, total * sizeof(double));
    const int nmax = n0 > n1 ? n0 : n1;
    double* re = (double*)malloc((size_t)nmax * sizeof(double));
    double* im = (double*)malloc((size_t)nmax * sizeof(double));
    for (int r = 0; r < n0; ++r) line_r2r(p->out + (size_t)r * n1, n1, 1, p->k1, re, im);
    for (int c = 0; c < n1; ++c) line_r2r(p->out + c, n0, n1, p->k0, re, im);
    free(re);
    free(im);
}
