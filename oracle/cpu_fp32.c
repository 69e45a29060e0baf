/*
 * cpu_fp32.c -- FP32 OpenMP transcription of the reference's operator
 * arithmetic, as a host-CPU program would run it: the timed CPU baseline of
 * the benchmark (its cpu_baseline entries and its reference arm).
 *
 * TEST AND MEASUREMENT INFRASTRUCTURE ONLY: nothing in the product package
 * links or calls it.  It is not the parity checker either (oracle.c, FP64, is):
 * it keeps the reference's single precision so that its speed is that of the
 * reference's algorithm on host cores.
 *
 * Transcribed steps, each in float as the reference computes it:
 *   - ray table: GenerateRayTraceMap_FB_ReconImage_OneView_kernel
 *     (FP/transform.cu:64-101): ray angle beta + left + (i+1/2) dcol, distance
 *     R/dx*sin(gamma) to the isocentre, chord of the FOV circle, n =
 *     floor(chord / 0.125f), start shifted by rfov/dx into texture coordinates;
 *   - ray march: RayTrace_ReconImage_OneView_kernel (FP/transform.cu:103-146):
 *     the sum of n bilinear clamp-to-edge samples at start + k step (texel
 *     centres at +1/2, FP/transform.cu:224-227), times 0.125 dx.  Weights are
 *     exact FP32 (the texture unit's are 8-bit);
 *   - pixel-driven BP: BackProjOneView_fan_curve_kernel (BP/transform.cu:67-95):
 *     U = R + x c + y s, t = -x s + y c with (s, c) = (-sin beta, -cos beta),
 *     col = (atanf(t/U) - left)/dcol + shift, added when 0 < col < C; the
 *     weighted form (FBP/transform.cu:61-89) multiplies by 1/(U^2 + t^2);
 *   - ramp filter: the Hsieh h'' taps times R d_angle dcol
 *     (FBP/transform.cu:149-162) and the middle C outputs of the full linear
 *     convolution of each row with them, computed directly in O(C^2)
 *     (ippsConv_32f, FBP/transform.cu:166-174).
 * OpenMP parallelises rays (FP), image rows (BP) and detector rows (filter).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define CPU_PI_F 3.14159265359f /* FP/transform.h:1 */
#define CPU_STEP 0.125f         /* FP/transform.cu:10 */

/* The decoded op attributes (the layout of ct_fan_geom / orc_geom). */
typedef struct cpu_geom {
    float sdd, sid;
    int32_t n_views;
    float full_angle;
    int32_t n_cols, nx, ny;
    float rfov, shift;
    int32_t n_slices;
    float det_bottom, drow, dz;
    float d_angle, dx, dy, xmin, ymin, dcol, left, start_angle;
} cpu_geom;

int cpu_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* tex2D(imgTexture2D, x, y) with linear filtering and clamp addressing */
static inline float bilerp(const float *im, int nx, int ny, float x, float y) {
    /* samples lie inside the FOV circle, so x - 1/2 > -1: floor by truncation */
    const float xb = x - 0.5f, yb = y - 0.5f;
    const int i = (int)(xb + 1.0f) - 1, j = (int)(yb + 1.0f) - 1;
    const float ax = xb - (float)i, ay = yb - (float)j;
    const int i0 = i < 0 ? 0 : (i > nx - 1 ? nx - 1 : i);
    const int i1 = i + 1 < 0 ? 0 : (i + 1 > nx - 1 ? nx - 1 : i + 1);
    const int j0 = j < 0 ? 0 : (j > ny - 1 ? ny - 1 : j);
    const int j1 = j + 1 < 0 ? 0 : (j + 1 > ny - 1 ? ny - 1 : j + 1);
    const float *r0 = im + (size_t)j0 * nx, *r1 = im + (size_t)j1 * nx;
    const float a = r0[i0] + ax * (r0[i1] - r0[i0]);
    const float b = r1[i0] + ax * (r1[i1] - r1[i0]);
    return a + ay * (b - a);
}

/* Forward projection of `batch` slices [batch][ny][nx] over the views
 * view0 .. view0 + n_views - 1 of `angles`; sino is [batch][n_views][n_cols]. */
void cpu_fp_fan(const cpu_geom *g, const float *angles, int view0, int n_views, const float *img,
                float *sino, int batch) {
    const int C = g->n_cols, nx = g->nx, ny = g->ny;
    const float Rp = g->sid / g->dx, rp = g->rfov / g->dx; /* (FP/transform.cu:239) */
    const float scale = CPU_STEP * g->dx;
    const long rays = (long)n_views * C;
#pragma omp parallel for schedule(dynamic, 64)
    for (long r = 0; r < rays; ++r) {
        const int v = (int)(r / C), i = (int)(r % C);
        const float ang = angles[view0 + v];
        /* fAngle + fColMin + (i + 0.5f) * fDeltaCol, evaluated left to right */
        const float ray_ang = ang + g->left + ((float)i + 0.5f) * g->dcol;
        const float sa = sinf(ray_ang), ca = cosf(ray_ang);
        const float d = Rp * sinf(g->left + ((float)i + 0.5f) * g->dcol);
        const float x1 = -sqrtf(rp * rp - d * d), x2 = -x1, y1 = -d, y2 = -d;
        const float p1x = x1 * ca - y1 * sa, p1y = x1 * sa + y1 * ca;
        const float p2x = x2 * ca - y2 * sa, p2y = x2 * sa + y2 * ca;
        const float dist = (float)sqrt((double)((p1x - p2x) * (p1x - p2x) +
                                                (p1y - p2y) * (p1y - p2y)));
        const float q = floorf(dist / CPU_STEP);
        const int n = q == q ? (int)q : 0; /* a ray missing the FOV: NaN -> 0 samples */
        const float sx = n > 0 ? (p2x - p1x) / (float)n : 0.0f;
        const float sy = n > 0 ? (p2y - p1y) / (float)n : 0.0f;
        const float x0 = p1x + rp, y0 = p1y + rp;
        for (int b = 0; b < batch; ++b) {
            const float *im = img + (size_t)b * nx * ny;
            float acc = 0.0f;
            for (int k = 0; k < n; ++k) acc += bilerp(im, nx, ny, x0 + k * sx, y0 + k * sy);
            sino[((size_t)b * n_views + v) * C + i] = acc * scale;
        }
    }
}

/* Pixel-driven backprojection of sino [batch][n_views][n_cols] (views
 * view0 .. view0 + n_views - 1 of `angles`) into img [batch][ny][nx];
 * weighted != 0 multiplies by 1/(U^2 + t^2) (FBP). */
void cpu_bp_fan(const cpu_geom *g, const float *angles, int view0, int n_views,
                const float *sino, float *img, int batch, int weighted) {
    const int C = g->n_cols, nx = g->nx, ny = g->ny;
    const float r2 = g->rfov * g->rfov;
    float *sn = (float *)malloc(sizeof(float) * 2 * n_views);
    for (int v = 0; v < n_views; ++v) {
        sn[2 * v] = -sinf(angles[view0 + v]);
        sn[2 * v + 1] = -cosf(angles[view0 + v]);
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (long bj = 0; bj < (long)batch * ny; ++bj) {
        const int b = (int)(bj / ny), j = (int)(bj % ny);
        float *row = img + ((size_t)b * ny + j) * nx;
        memset(row, 0, sizeof(float) * nx);
        const float y = g->ymin + g->dy * ((float)j + 0.5f);
        for (int v = 0; v < n_views; ++v) {
            const float s = sn[2 * v], c = sn[2 * v + 1];
            const float *sv = sino + ((size_t)b * n_views + v) * C;
            for (int i = 0; i < nx; ++i) {
                const float x = g->xmin + g->dx * ((float)i + 0.5f);
                if (x * x + y * y > r2) continue;
                const float U = g->sid + x * c + y * s;
                const float t = -x * s + y * c;
                const float col = (atanf(t / U) - g->left) / g->dcol + g->shift;
                if (!(col > 0.0f && col < (float)C)) continue;
                /* tex1D at col: texel centres at +1/2, clamp addressing */
                const float cb = col - 0.5f; /* > -1/2 */
                const int k = (int)(cb + 1.0f) - 1;
                const float f = cb - (float)k;
                const int k0 = k < 0 ? 0 : k, k1 = k + 1 > C - 1 ? C - 1 : k + 1;
                float val = sv[k0] + f * (sv[k1] - sv[k0]);
                if (weighted) val *= 1.0f / (U * U + t * t);
                row[i] += val;
            }
        }
    }
    free(sn);
}

/* The reference's Ram-Lak taps in float (FBP/transform.cu:149-162), index
 * n + C - 1 for n in [-(C-1), C-1]. */
void cpu_ramp_taps(const cpu_geom *g, float *taps) {
    const int C = g->n_cols;
    const float dc = g->dcol;
    for (int n = -C + 1; n <= C - 1; ++n) {
        float h;
        if (n == 0)
            h = 0.5f / (4 * dc * dc);
        else if (n % 2)
            h = -0.5f / (CPU_PI_F * CPU_PI_F * sinf(n * dc) * sinf(n * dc));
        else
            h = 0.0f;
        taps[n + C - 1] = h;
    }
    const float k = g->sid * g->d_angle * dc;
    for (int n = 0; n < 2 * C - 1; ++n) taps[n] *= k;
}

/* out[r][i] = sum_j in[r][j] taps[i - j + C - 1] for each of `rows` rows (the
 * middle C outputs of the full convolution), directly in O(C^2). */
void cpu_ramp_filter(const cpu_geom *g, const float *taps, const float *in, float *out,
                     long rows) {
    const int C = g->n_cols;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < rows; ++r) {
        const float *p = in + (size_t)r * C;
        float *q = out + (size_t)r * C;
        for (int i = 0; i < C; ++i) {
            const float *h = taps + i + C - 1; /* h[-j] = taps[i - j + C - 1] */
            float acc = 0.0f;
#pragma omp simd reduction(+ : acc)
            for (int j = 0; j < C; ++j) acc += p[j] * h[-j];
            q[i] = acc;
        }
    }
}

/* FBP: ramp filter of every row, then the weighted BP.  work holds
 * batch * n_views * n_cols floats. */
void cpu_fbp_fan(const cpu_geom *g, const float *angles, int view0, int n_views,
                 const float *sino, float *img, int batch, float *work) {
    float *taps = (float *)malloc(sizeof(float) * (2 * g->n_cols - 1));
    cpu_ramp_taps(g, taps);
    cpu_ramp_filter(g, taps, sino, work, (long)batch * n_views);
    cpu_bp_fan(g, angles, view0, n_views, work, img, batch, 1);
    free(taps);
}
