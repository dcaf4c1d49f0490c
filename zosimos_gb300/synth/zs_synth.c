/*
 * zs_synth.c -- seeded synthetic images for the benchmark workloads and the parity
 * tests (no image dataset exists for this path), generated on the host cores.
 *
 * The same counter-based scheme as zosimos_gb300/synthetic.py: every value is
 * splitmix64(key(seed, image, pixel, channel)), so any image of a batch is generated
 * independently and identically wherever it is made.  OpenMP over rows; no FMA
 * contraction (-ffp-contract=off), so x86_64 and aarch64 hosts agree.
 *
 * Not part of the executor: bench.py and the tests call it through ctypes to make
 * inputs.  Half-precision outputs are IEEE binary16 bit patterns, rounded to nearest
 * even directly from the double value (no double rounding through float).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define SM_GOLD 0x9E3779B97F4A7C15ull
#define SM_M1 0xBF58476D1CE4E5B9ull
#define SM_M2 0x94D049BB133111EBull

static uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + SM_GOLD;
    z = (z ^ (z >> 30)) * SM_M1;
    z = (z ^ (z >> 27)) * SM_M2;
    return z ^ (z >> 31);
}

static uint64_t key_base(int32_t seed, int32_t image) {
    return ((uint64_t)(seed & 0xFFFF) << 48) | ((uint64_t)(image & 0xFFFF) << 32);
}

/* IEEE binary16 bits of d, round to nearest even, subnormals kept. */
static uint16_t d2h(double d) {
    uint64_t x;
    memcpy(&x, &d, 8);
    const uint16_t sign = (uint16_t)((x >> 48) & 0x8000u);
    const uint64_t ax = x & 0x7FFFFFFFFFFFFFFFull;
    if (ax >= 0x7FF0000000000000ull) return (uint16_t)(sign | 0x7C00u | (ax > 0x7FF0000000000000ull ? 0x200u : 0u));
    const int e = (int)(ax >> 52) - 1023 + 15;
    uint64_t mant = ax & 0xFFFFFFFFFFFFFull;
    if (e >= 31) return (uint16_t)(sign | 0x7C00u);
    if (e <= 0) {
        if (e < -10) return sign;
        mant |= 1ull << 52;
        const int shift = 43 - e;
        uint64_t h = mant >> shift;
        const uint64_t rem = mant & ((1ull << shift) - 1ull), half = 1ull << (shift - 1);
        if (rem > half || (rem == half && (h & 1ull))) ++h;
        return (uint16_t)(sign | h);
    }
    uint64_t h = ((uint64_t)e << 10) | (mant >> 42);
    const uint64_t rem = mant & ((1ull << 42) - 1ull);
    if (rem > (1ull << 41) || (rem == (1ull << 41) && (h & 1ull))) ++h;
    return (uint16_t)(sign | h);
}

static double max1(double v) { return v > 1.0 ? v : 1.0; }

/* RGBA8 sRGB: R = x ramp, G = y ramp, B = diagonal ramp, each plus uniform integer noise in
 * [-noise, noise] (clamped), alpha uniform in [0, 255] (or 255).  out: h * w * 4 bytes. */
void zs_synth_srgb_gradient_noise(int32_t w, int32_t h, int32_t seed, int32_t image, int32_t noise,
                                  int32_t random_alpha, uint8_t *out) {
    const uint64_t base = key_base(seed, image), mod = (uint64_t)(2 * noise + 1);
    const double mx = max1((double)(w - 1)), my = max1((double)(h - 1)), md = max1((double)(w + h - 2));
#pragma omp parallel for schedule(static)
    for (int32_t y = 0; y < h; y++) {
        for (int32_t x = 0; x < w; x++) {
            const uint64_t px = (uint64_t)y * (uint64_t)w + (uint64_t)x;
            const double ramp[3] = {nearbyint(255.0 * x / mx), nearbyint(255.0 * y / my),
                                    nearbyint(255.0 * (double)(x + y) / md)};
            uint8_t *o = out + px * 4;
            for (int c = 0; c < 3; c++) {
                const uint64_t z = splitmix64(base ^ (px * 4 + (uint64_t)c));
                const int64_t v = (int64_t)ramp[c] + (int64_t)(z % mod) - noise;
                o[c] = (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
            }
            o[3] = random_alpha ? (uint8_t)(splitmix64(base ^ (px * 4 + 3)) & 255u) : 255;
        }
    }
}

/* Linear colour of pixel (x, y) channel c: ramp + sigma * N(0, 1) (Box-Muller), clamped. */
static double gauss_value(uint64_t base, uint64_t px, int c, double ramp, double sigma) {
    const uint64_t z1 = splitmix64(base ^ (px * 4 + (uint64_t)c)), z2 = splitmix64(z1);
    const double u1 = ((double)(z1 >> 11) + 1.0) / 9007199254740992.0;
    const double u2 = (double)(z2 >> 11) / 9007199254740992.0;
    const double g = sqrt(-2.0 * log(u1)) * cos(2.0 * 3.141592653589793 * u2);
    const double v = ramp + sigma * g;
    return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
}

/* Linear RGBA16F: gradient ramps plus Gaussian noise (sigma), clamped to [0, 1], alpha 1.
 * out: h * w * 4 binary16 values. */
void zs_synth_linear_gradient_gauss(int32_t w, int32_t h, int32_t seed, int32_t image, double sigma,
                                    uint16_t *out) {
    const uint64_t base = key_base(seed, image);
    const double mx = max1((double)(w - 1)), my = max1((double)(h - 1)), md = max1((double)(w + h - 2));
#pragma omp parallel for schedule(static)
    for (int32_t y = 0; y < h; y++) {
        for (int32_t x = 0; x < w; x++) {
            const uint64_t px = (uint64_t)y * (uint64_t)w + (uint64_t)x;
            const double ramp[3] = {(double)x / mx, (double)y / my, (double)(x + y) / md};
            uint16_t *o = out + px * 4;
            for (int c = 0; c < 3; c++) o[c] = d2h(gauss_value(base, px, c, ramp[c], sigma));
            o[3] = 0x3C00u;
        }
    }
}

/* Premultiplied linear RGBA16F: the gradient + Gaussian-noise colour (sigma 0.05), alpha the
 * clamped sum of `blobs` 2D Gaussian blobs whose centre, width (sigma in [128, 768] px at
 * 4096 px, scaled with the image) and amplitude ([0.3, 1]) come from the uniform stream of
 * image ^ 0x8000, channel 7.  out: h * w * 4 binary16 values. */
void zs_synth_premultiplied_layer(int32_t w, int32_t h, int32_t seed, int32_t image, int32_t blobs,
                                  uint16_t *out) {
    const uint64_t base = key_base(seed, image), ubase = key_base(seed, image ^ 0x8000);
    const double mx = max1((double)(w - 1)), my = max1((double)(h - 1)), md = max1((double)(w + h - 2));
    const double scale = (double)(w > h ? w : h) / 4096.0;
    double cx[64], cy[64], s2[64], amp[64];
    if (blobs > 64) blobs = 64;
    for (int b = 0; b < blobs; b++) {
        double u[4];
        for (int k = 0; k < 4; k++)
            u[k] = (double)(splitmix64(ubase ^ ((uint64_t)(4 * b + k) * 4 + 7)) >> 11) / 9007199254740992.0;
        cx[b] = u[0] * w;
        cy[b] = u[1] * h;
        const double sigma = (128.0 + 640.0 * u[2]) * scale;
        s2[b] = 2.0 * sigma * sigma;
        amp[b] = 0.3 + 0.7 * u[3];
    }
#pragma omp parallel for schedule(static)
    for (int32_t y = 0; y < h; y++) {
        for (int32_t x = 0; x < w; x++) {
            const uint64_t px = (uint64_t)y * (uint64_t)w + (uint64_t)x;
            double alpha = 0.0;
            for (int b = 0; b < blobs; b++) {
                const double dx = (double)x - cx[b], dy = (double)y - cy[b];
                alpha += amp[b] * exp(-(dx * dx + dy * dy) / s2[b]);
            }
            alpha = alpha < 0.0 ? 0.0 : (alpha > 1.0 ? 1.0 : alpha);
            const double ramp[3] = {(double)x / mx, (double)y / my, (double)(x + y) / md};
            uint16_t *o = out + px * 4;
            for (int c = 0; c < 3; c++) o[c] = d2h(gauss_value(base, px, c, ramp[c], 0.05) * alpha);
            o[3] = d2h(alpha);
        }
    }
}
