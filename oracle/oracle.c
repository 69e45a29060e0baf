/*
 * oracle.c -- FP64 CPU restatement of FanBeamCTRecon_TensorflowOp's four
 * operators.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and
 * the CPU-baseline leg of the benchmark call it as the checker; no product
 * code path links or executes it.
 *
 * Parity status: PINNED to the reference's own ops, executed.  The reference
 * cannot be built for the GPU here (legacy texture references do not compile
 * with CUDA 13; TensorFlow, Intel IPP and helper_cuda.h are absent), so its op
 * wrappers and CUDA sources are compiled for the host against stand-ins for
 * those three (build_ref.py, refexec/) and executed; the outputs are the
 * golden vectors of tests/golden/reference_ops.npz.  With the texture unit's
 * weights (texture_rule.h) this restatement meets them within 2e-6 (FP),
 * 1e-6 (BP) and 5e-5 (FBP, FDK) relative L2.  Further pins: the reference's
 * Python geometry packing (utils.py, config.py) executed for golden
 * parameter/angle vectors, exact known answers of the discrete operators,
 * analytic ellipse line integrals, and FP64 adjoint identities.
 *
 * Every function follows the reference's arithmetic in double precision,
 * citing the file:line it restates.  Geometry decoding stays in float, as the
 * op constructors do it, because those floats are the op's attributes.
 *
 * Optional texture emulation (orc_set_texture_emulation(1)) applies the GPU
 * texture unit's linear-filter weights (texture_rule.h: fractions rounded to
 * 1/256, the 2-D far-corner weight rounded to 1/256) to bound how far the
 * reference's texture-unit outputs sit from exact bilinear interpolation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "texture_rule.h"

#define ORC_PI_F 3.14159265359f /* FP/transform.h:1 */
#define ORC_STEP 0.125          /* FP/transform.cu:10 */

typedef struct orc_geom {
    float sdd, sid;
    int32_t n_views;
    float full_angle;
    int32_t n_cols, nx, ny;
    float rfov, shift;
    int32_t n_slices;
    float det_bottom, drow, dz;
    float d_angle, dx, dy, xmin, ymin, dcol, left, start_angle;
} orc_geom;

static int g_tex8 = 0;

void orc_set_texture_emulation(int on) { g_tex8 = on ? 1 : 0; }

static double frac_w(double f) {
    /* 8 fractional bits, round to nearest (texture filtering precision) */
    return g_tex8 ? floor(f * 256.0 + 0.5) / 256.0 : f;
}

/* FP/transform.cc:59-76 (FDK/FBP.cc:61-84 for the last three) */
int orc_decode_param16(const float *p, orc_geom *g) {
    memset(g, 0, sizeof(*g));
    if (!isfinite(p[2]) || !isfinite(p[4]) || !isfinite(p[5]) || !isfinite(p[6]) ||
        !isfinite(p[11]))
        return 1;
    g->sdd = p[0];
    g->sid = p[1];
    g->n_views = (int32_t)p[2];
    g->full_angle = p[3];
    g->n_cols = (int32_t)p[4];
    g->nx = (int32_t)p[5];
    g->ny = (int32_t)p[6];
    g->rfov = p[7];
    g->shift = p[9];
    g->n_slices = (int32_t)p[11];
    g->det_bottom = p[13];
    g->drow = p[14];
    g->dz = p[15];
    if (g->n_views <= 0 || g->nx <= 0 || g->ny <= 0) return 1;
    {
        float a = g->full_angle / (float)g->n_views;
        a = a * ORC_PI_F;
        g->d_angle = a / 180.0f;
    }
    {
        float two_r = 2.0f * g->rfov;
        float hx, hy;
        g->dx = two_r / (float)g->nx;
        g->dy = two_r / (float)g->ny;
        hx = -0.5f * (float)g->nx;
        hy = -0.5f * (float)g->ny;
        g->xmin = hx * g->dx;
        g->ymin = hy * g->dy;
    }
    {
        float t = p[8] * ORC_PI_F;
        g->dcol = t / 180.0f;
        t = p[10] * ORC_PI_F;
        g->left = t / 180.0f;
        t = p[12] * ORC_PI_F;
        g->start_angle = t / 180.0f;
    }
    return 0;
}

/* GenerateRayTraceMap_FB_ReconImage_OneView_kernel, FP/transform.cu:64-101:
 * ray angle beta + left + (i+1/2) dcol; distance R/dx*sin(gamma) of the ray
 * from the isocentre; intersections with the FOV circle of radius rfov/dx;
 * n = floor(chord/0.125); start shifted by rfov/dx into texture coordinates.
 * A ray missing the circle gets n = 0 (the reference's sqrtf(negative) = NaN
 * converts to 0 samples). */
void orc_ray_table(const orc_geom *g, const float *angles, double *ray, int32_t *nsamp) {
    const int V = g->n_views, C = g->n_cols;
    const double dx = g->dx;
    const double src = (double)g->sid / dx, fov = (double)g->rfov / dx;
    const double left = g->left, dcol = g->dcol;
#pragma omp parallel for schedule(static)
    for (int v = 0; v < V; ++v) {
        const double beta = angles[v];
        for (int i = 0; i < C; ++i) {
            const size_t r = (size_t)v * C + i;
            double *q = ray + 4 * r;
            const double gam = left + (i + 0.5) * dcol;
            const double th = beta + gam;
            const double sn = sin(th), cs = cos(th);
            const double dist = src * sin(gam);
            const double h = fov * fov - dist * dist;
            double x1, x2, y1, y2, ax, ay, bx, by, L, nn;
            q[0] = q[1] = q[2] = q[3] = 0.0;
            nsamp[r] = 0;
            if (!(h > 0.0)) continue;
            x1 = -sqrt(h);
            x2 = -x1;
            y1 = -dist;
            y2 = -dist;
            ax = x1 * cs - y1 * sn;
            ay = x1 * sn + y1 * cs;
            bx = x2 * cs - y2 * sn;
            by = x2 * sn + y2 * cs;
            L = sqrt((ax - bx) * (ax - bx) + (ay - by) * (ay - by));
            nn = floor(L / ORC_STEP);
            if (!(nn >= 1.0)) continue;
            nsamp[r] = (int32_t)nn;
            q[0] = ax + fov;
            q[1] = ay + fov;
            q[2] = (bx - ax) / nn;
            q[3] = (by - ay) / nn;
        }
    }
}

/* tex2D with cudaFilterModeLinear + cudaAddressModeClamp on an nx-by-ny float
 * array: texel (i, j) centred at (i+1/2, j+1/2), clamp-to-edge taps.  With
 * texture emulation on, the weights are the texture unit's (texture_rule.h). */
typedef struct tap4 {
    int i0, i1, j0, j1;
    double w00, w10, w01, w11;
} tap4;

static tap4 bilinear_taps(int nx, int ny, double x, double y) {
    tap4 t;
    const double xb = x - 0.5, yb = y - 0.5;
    const double fx = floor(xb), fy = floor(yb);
    const double ax = frac_w(xb - fx), ay = frac_w(yb - fy);
    const int i = (int)fx, j = (int)fy;
    t.i0 = i < 0 ? 0 : (i > nx - 1 ? nx - 1 : i);
    t.i1 = i + 1 < 0 ? 0 : (i + 1 > nx - 1 ? nx - 1 : i + 1);
    t.j0 = j < 0 ? 0 : (j > ny - 1 ? ny - 1 : j);
    t.j1 = j + 1 < 0 ? 0 : (j + 1 > ny - 1 ? ny - 1 : j + 1);
    if (g_tex8) {
        int k[4];
        ctex_weights2d((int)(ax * 256.0), (int)(ay * 256.0), k);
        t.w00 = k[0] / 256.0;
        t.w10 = k[1] / 256.0;
        t.w01 = k[2] / 256.0;
        t.w11 = k[3] / 256.0;
        return t;
    }
    t.w00 = (1.0 - ax) * (1.0 - ay);
    t.w10 = ax * (1.0 - ay);
    t.w01 = (1.0 - ax) * ay;
    t.w11 = ax * ay;
    return t;
}

/* The texture unit's filter (texture_rule.h) on n coordinates, so that the
 * tests can hold the rule against fetches measured on the GPU. */
void orc_tex_fetch1d(const float *t, int w, const float *x, float *out, int n) {
    for (int k = 0; k < n; ++k) out[k] = ctex_fetch1d(t, w, x[k]);
}
void orc_tex_fetch2d(const float *t, int w, int h, const float *x, const float *y, float *out,
                     int n) {
    for (int k = 0; k < n; ++k) out[k] = ctex_fetch2d(t, w, h, x[k], y[k]);
}

/* RayTrace_ReconImage_OneView_kernel, FP/transform.cu:103-146:
 * p = 0.125 * dx * sum_{k<n} tex2D(start + k*step). */
void orc_fp_fan(const orc_geom *g, const float *angles, const double *img, double *sino,
                int batch) {
    const int V = g->n_views, C = g->n_cols, nx = g->nx, ny = g->ny;
    const size_t R = (size_t)V * C;
    double *ray = (double *)malloc(sizeof(double) * 4 * R);
    int32_t *ns = (int32_t *)malloc(sizeof(int32_t) * R);
    const double w = ORC_STEP * (double)g->dx;
    orc_ray_table(g, angles, ray, ns);
    for (int b = 0; b < batch; ++b) {
        const double *im = img + (size_t)b * nx * ny;
        double *out = sino + (size_t)b * R;
#pragma omp parallel for schedule(dynamic, 64)
        for (long r = 0; r < (long)R; ++r) {
            const double *q = ray + 4 * r;
            double acc = 0.0;
            for (int k = 0; k < ns[r]; ++k) {
                const tap4 t = bilinear_taps(nx, ny, q[0] + k * q[2], q[1] + k * q[3]);
                acc += t.w00 * im[t.j0 * nx + t.i0] + t.w10 * im[t.j0 * nx + t.i1] +
                       t.w01 * im[t.j1 * nx + t.i0] + t.w11 * im[t.j1 * nx + t.i1];
            }
            out[r] = acc * w;
        }
    }
    free(ray);
    free(ns);
}

/* Exact transpose of orc_fp_fan (no reference counterpart). */
void orc_fp_fan_adjoint(const orc_geom *g, const float *angles, const double *sino, double *img,
                        int batch) {
    const int V = g->n_views, C = g->n_cols, nx = g->nx, ny = g->ny;
    const size_t R = (size_t)V * C, N = (size_t)nx * ny;
    double *ray = (double *)malloc(sizeof(double) * 4 * R);
    int32_t *ns = (int32_t *)malloc(sizeof(int32_t) * R);
    const double w = ORC_STEP * (double)g->dx;
    orc_ray_table(g, angles, ray, ns);
    memset(img, 0, sizeof(double) * N * batch);
    for (int b = 0; b < batch; ++b) {
        const double *in = sino + (size_t)b * R;
        double *im = img + (size_t)b * N;
        /* each thread scatters into a private image; the images are summed */
#pragma omp parallel
        {
            double *priv = (double *)calloc(N, sizeof(double));
#pragma omp for schedule(dynamic, 64)
            for (long r = 0; r < (long)R; ++r) {
                const double *q = ray + 4 * r;
                const double val = in[r] * w;
                if (val == 0.0) continue;
                for (int k = 0; k < ns[r]; ++k) {
                    const tap4 t = bilinear_taps(nx, ny, q[0] + k * q[2], q[1] + k * q[3]);
                    priv[t.j0 * nx + t.i0] += val * t.w00;
                    priv[t.j0 * nx + t.i1] += val * t.w10;
                    priv[t.j1 * nx + t.i0] += val * t.w01;
                    priv[t.j1 * nx + t.i1] += val * t.w11;
                }
            }
#pragma omp critical
            for (size_t p = 0; p < N; ++p) im[p] += priv[p];
            free(priv);
        }
    }
    free(ray);
    free(ns);
}

/* Pixel geometry shared by the BP family (BP/transform.cu:76-92,116;
 * FBP/transform.cu:70-87; FDK/GPURecon_GPU.cu:25-49). Returns 1 when the
 * detector coordinate lies in (0, C) and fills the taps/weight. */
static int bp_col(const orc_geom *g, double x, double y, double c, double s, int *i0, int *i1,
                  double *f, double *U_out, double *t_out) {
    const double U = (double)g->sid + x * c + y * s;
    const double t = -x * s + y * c;
    const double col = (atan(t / U) - (double)g->left) / (double)g->dcol + (double)g->shift;
    *U_out = U;
    *t_out = t;
    if (!(col > 0.0 && col < (double)g->n_cols)) return 0;
    {
        const double cb = col - 0.5;
        const double fi = floor(cb);
        const int i = (int)fi;
        *f = frac_w(cb - fi);
        *i0 = i < 0 ? 0 : i;
        *i1 = i + 1 > g->n_cols - 1 ? g->n_cols - 1 : i + 1;
    }
    return 1;
}

/* Weights of a (column, row) sample whose fractions f, fr came through frac_w:
 * w[0] (row r0, col i0), w[1] (r0, i1), w[2] (r1, i0), w[3] (r1, i1).  Exact
 * bilinear, or with texture emulation the texture unit's (texture_rule.h). */
static void bilinear_w(double f, double fr, double w[4]) {
    if (g_tex8) {
        int k[4];
        ctex_weights2d((int)(f * 256.0), (int)(fr * 256.0), k);
        for (int n = 0; n < 4; ++n) w[n] = k[n] / 256.0;
        return;
    }
    w[0] = (1.0 - f) * (1.0 - fr);
    w[1] = f * (1.0 - fr);
    w[2] = (1.0 - f) * fr;
    w[3] = f * fr;
}

/* BackProjOneView_fan_curve_kernel summed over views (BP/transform.cu:67-95,
 * 110-119); weighted != 0 adds the 1/(U^2+t^2) factor of FBP/transform.cu:78. */
void orc_bp_fan(const orc_geom *g, const float *angles, const double *sino, double *img,
                int batch, int weighted) {
    const int V = g->n_views, C = g->n_cols, nx = g->nx, ny = g->ny;
    const double r2 = (double)g->rfov * (double)g->rfov;
    for (int b = 0; b < batch; ++b) {
        const double *sb = sino + (size_t)b * V * C;
        double *im = img + (size_t)b * nx * ny;
#pragma omp parallel for schedule(dynamic, 4)
        for (int j = 0; j < ny; ++j) {
            const double y = (double)g->ymin + (double)g->dy * (j + 0.5);
            for (int i = 0; i < nx; ++i) {
                const double x = (double)g->xmin + (double)g->dx * (i + 0.5);
                double acc = 0.0;
                if (x * x + y * y <= r2) {
                    for (int v = 0; v < V; ++v) {
                        const double beta = angles[v];
                        const double c = -cos(beta), s = -sin(beta);
                        int i0, i1;
                        double f, U, t;
                        if (bp_col(g, x, y, c, s, &i0, &i1, &f, &U, &t)) {
                            const double *row = sb + (size_t)v * C;
                            double val = (1.0 - f) * row[i0] + f * row[i1];
                            if (weighted) val *= 1.0 / (U * U + t * t);
                            acc += val;
                        }
                    }
                }
                im[(size_t)j * nx + i] = acc;
            }
        }
    }
}

/* Transpose of orc_bp_fan (no reference counterpart). */
void orc_bp_fan_transpose(const orc_geom *g, const float *angles, const double *img,
                          double *sino, int batch, int weighted) {
    const int V = g->n_views, C = g->n_cols, nx = g->nx, ny = g->ny;
    const double r2 = (double)g->rfov * (double)g->rfov;
    memset(sino, 0, sizeof(double) * (size_t)batch * V * C);
    for (int b = 0; b < batch; ++b) {
        const double *im = img + (size_t)b * nx * ny;
        double *sb = sino + (size_t)b * V * C;
#pragma omp parallel for schedule(dynamic, 4)
        for (int v = 0; v < V; ++v) {
            const double beta = angles[v];
            const double c = -cos(beta), s = -sin(beta);
            double *row = sb + (size_t)v * C;
            for (int j = 0; j < ny; ++j) {
                const double y = (double)g->ymin + (double)g->dy * (j + 0.5);
                for (int i = 0; i < nx; ++i) {
                    const double x = (double)g->xmin + (double)g->dx * (i + 0.5);
                    int i0, i1;
                    double f, U, t, val;
                    if (!(x * x + y * y <= r2)) continue;
                    val = im[(size_t)j * nx + i];
                    if (val == 0.0) continue;
                    if (!bp_col(g, x, y, c, s, &i0, &i1, &f, &U, &t)) continue;
                    if (weighted) val *= 1.0 / (U * U + t * t);
                    row[i0] += val * (1.0 - f);
                    row[i1] += val * f;
                }
            }
        }
    }
}

/* Ramp taps, index n + C - 1 (FBP/transform.cu:149-162; FDK/GPURecon_GPU.cu:
 * 184-200).  window 0: the reference's Hsieh h'' Ram-Lak form with the 0.5
 * factor; window 1: Shepp-Logan 0.5*2/(pi^2 dcol^2 (1-4n^2)) times
 * (n dcol/sin(n dcol))^2.  Scaled by R * d_angle * dcol. */
void orc_ramp_taps(const orc_geom *g, int window, double *taps) {
    const int C = g->n_cols;
    const double pi = (double)ORC_PI_F, dc = g->dcol;
    const double scale = (double)g->sid * (double)g->d_angle * dc;
    for (int n = -(C - 1); n <= C - 1; ++n) {
        double h;
        if (window == 1) {
            if (n == 0) {
                h = 0.5 * 2.0 / (pi * pi * dc * dc);
            } else {
                const double s = sin(n * dc);
                h = 0.5 * 2.0 * (double)n * (double)n /
                    (pi * pi * s * s * (1.0 - 4.0 * (double)n * (double)n));
            }
        } else if (n == 0) {
            h = 0.5 / (4.0 * dc * dc);
        } else if (n % 2 != 0) {
            const double s = sin(n * dc);
            h = -0.5 / (pi * pi * s * s);
        } else {
            h = 0.0;
        }
        taps[n + C - 1] = h * scale;
    }
}

/* ippsConv_32f full linear convolution of each row with the 2C-1 taps,
 * keeping samples C-1 .. 2C-2 (FBP/transform.cu:166-174):
 * q[i] = sum_j p[j] * taps[i - j + C - 1]. */
void orc_ramp_filter(const orc_geom *g, int window, const double *in, double *out, long rows) {
    const int C = g->n_cols;
    double *taps = (double *)malloc(sizeof(double) * (2 * (size_t)C - 1));
    orc_ramp_taps(g, window, taps);
#pragma omp parallel for schedule(static)
    for (long r = 0; r < rows; ++r) {
        const double *p = in + (size_t)r * C;
        double *q = out + (size_t)r * C;
        for (int i = 0; i < C; ++i) {
            double acc = 0.0;
            for (int j = 0; j < C; ++j) acc += p[j] * taps[i - j + C - 1];
            q[i] = acc;
        }
    }
    free(taps);
}

/* Parker short-scan weight (Parker, Med. Phys. 9(2), 1982), written as the
 * product of a rising and a falling smooth step S(u) = sin^2(pi u / 2) on
 * [0, 1] (0 below, 1 above): w = S(beta / (2 (G - gam))) *
 * S((pi + 2 G - beta) / (2 (G + gam))), which equals the piecewise form for
 * fans narrower than pi and is 0 outside [0, pi + 2 G]. */
#define ORC_PI_D 3.14159265358979323846

static double orc_smooth_step(double u) {
    if (u <= 0.0) return 0.0;
    if (u >= 1.0) return 1.0;
    const double s = sin(0.5 * ORC_PI_D * u);
    return s * s;
}

double orc_parker_weight(double beta, double gam, double G) {
    if (beta < 0.0 || beta > ORC_PI_D + 2.0 * G) return 0.0;
    return orc_smooth_step(beta / (2.0 * (G - gam))) *
           orc_smooth_step((ORC_PI_D + 2.0 * G - beta) / (2.0 * (G + gam)));
}

/* Doubled Parker weights per (view, channel): beta from angles[0] (mirrored
 * for decreasing angles), gam = left + (i + 1/2 - shift) dcol, G the outer
 * edge of the outermost channel.  The 2 undoes the 0.5 of the ramp taps. */
void orc_parker_weights(const orc_geom *g, const float *angles, double *w) {
    const int V = g->n_views, C = g->n_cols;
    const double dc = g->dcol;
    const double dir = (V > 1 && angles[V - 1] < angles[0]) ? -1.0 : 1.0;
    double G = 0.0;
    for (int i = 0; i < C; ++i) {
        const double a = fabs((double)g->left + (i + 0.5 - (double)g->shift) * dc) + 0.5 * dc;
        if (a > G) G = a;
    }
    for (int v = 0; v < V; ++v)
        for (int i = 0; i < C; ++i) {
            const double beta = dir * ((double)angles[v] - (double)angles[0]);
            const double gam = dir * ((double)g->left + (i + 0.5 - (double)g->shift) * dc);
            w[(size_t)v * C + i] = 2.0 * orc_parker_weight(beta, gam, G);
        }
}

/* backproject_fan_curve of FBP/transform.cu:117-201: filter, then weighted BP. */
void orc_fbp_fan(const orc_geom *g, const float *angles, int window, const double *sino,
                 double *img, int batch) {
    const size_t n = (size_t)batch * g->n_views * g->n_cols;
    double *tmp = (double *)malloc(sizeof(double) * (n ? n : 1));
    orc_ramp_filter(g, window, sino, tmp, (long)batch * g->n_views);
    orc_bp_fan(g, angles, tmp, img, batch, 1);
    free(tmp);
}

/* Transpose of orc_fbp_fan: weighted-BP transpose, then the (symmetric) filter. */
void orc_fbp_fan_adjoint(const orc_geom *g, const float *angles, int window, const double *img,
                         double *sino, int batch) {
    const size_t n = (size_t)batch * g->n_views * g->n_cols;
    double *tmp = (double *)malloc(sizeof(double) * (n ? n : 1));
    orc_bp_fan_transpose(g, angles, img, tmp, batch, 1);
    orc_ramp_filter(g, window, tmp, sino, (long)batch * g->n_views);
    free(tmp);
}

/* The "BackProjection" op (FDK/FBP.cc:61-110 -> BP_One_Rot_3D_GPU,
 * FDK/GPURecon_GPU.cu:163-268): filter each (view, row), then per view the
 * CB_EA kernel (:15-50) over nz slices with row index
 * ((z - z_src) * D / U - det_bottom) / drow on an n_rows-high view texture
 * (clamped), weight 1/(U^2+t^2).  The op fixes nz = n_rows = 1
 * (FDK/FBP.cc:85,98), zmin = -dz/2, z_src = 0 (FDK/GPURecon_GPU.cu:226). */
void orc_fdk_bp(const orc_geom *g, const float *angles, int window, const double *sino,
                double *img, int batch) {
    const int V = g->n_views, C = g->n_cols, nx = g->nx, ny = g->ny;
    const int n_rows = 1, nz = 1;
    const float zmin = -0.5f * g->dz * (float)nz;
    const double r2 = (double)g->rfov * (double)g->rfov;
    const size_t n = (size_t)batch * V * C;
    double *filt = (double *)malloc(sizeof(double) * (n ? n : 1));
    orc_ramp_filter(g, window, sino, filt, (long)batch * V * n_rows);
    for (int b = 0; b < batch; ++b) {
        const double *sb = filt + (size_t)b * V * C * n_rows;
        double *im = img + (size_t)b * nx * ny * nz;
#pragma omp parallel for schedule(dynamic, 4)
        for (int j = 0; j < ny; ++j) {
            const double y = (double)g->ymin + (double)g->dy * (j + 0.5);
            for (int i = 0; i < nx; ++i) {
                const double x = (double)g->xmin + (double)g->dx * (i + 0.5);
                for (int k = 0; k < nz; ++k) {
                    double acc = 0.0;
                    const double zk = (double)zmin + (double)g->dz * (k + 0.5);
                    if (x * x + y * y <= r2) {
                        for (int v = 0; v < V; ++v) {
                            const double beta = angles[v];
                            const double c = -cos(beta), s = -sin(beta);
                            int i0, i1;
                            double f, U, t;
                            if (bp_col(g, x, y, c, s, &i0, &i1, &f, &U, &t)) {
                                const double row = ((zk - 0.0) * (double)g->sdd / U -
                                                    (double)g->det_bottom) /
                                                   (double)g->drow;
                                const double rb = row - 0.5, rf = floor(rb);
                                const double fr = frac_w(rb - rf);
                                const int r0 = (int)rf;
                                const int ra = r0 < 0 ? 0 : (r0 > n_rows - 1 ? n_rows - 1 : r0);
                                const int rc =
                                    r0 + 1 < 0 ? 0 : (r0 + 1 > n_rows - 1 ? n_rows - 1 : r0 + 1);
                                const double *va = sb + ((size_t)v * n_rows + ra) * C;
                                const double *vc = sb + ((size_t)v * n_rows + rc) * C;
                                double w[4];
                                bilinear_w(f, fr, w);
                                acc += (w[0] * va[i0] + w[1] * va[i1] + w[2] * vc[i0] +
                                        w[3] * vc[i1]) /
                                       (U * U + t * t);
                            }
                        }
                    }
                    im[((size_t)k * ny + j) * nx + i] = acc;
                }
            }
        }
    }
    free(filt);
}

/* ---- cone beam ------------------------------------------------------------
 * Volume [B][nz][ny][nx]; projections [B][V][n_rows][C] (the reference's view
 * layout, FDK/GPURecon_GPU.cu:211: view * nCols * nRows + row * nCols).
 * Voxel centres: x = xmin + dx(i+1/2), y likewise, z = zmin + dz(k+1/2) with
 * zmin = -dz*nz/2 (FDK/FBP.cc:86); the source orbits at z = 0
 * (FDK/GPURecon_GPU.cu:226). */

/* CB_EA backprojection, FDK/GPURecon_GPU.cu:25-49, for any nz and n_rows:
 * per voxel in the FOV disc and view, col = (atan(t/U) - left)/dcol + shift
 * (0 < col < C), row = (z * D / U - det_bottom) / drow, bilinear clamped
 * sample of the [n_rows][C] view at (col, row), weight 1/(U^2+t^2). */
static void cone_bp_impl(const orc_geom *g, int n_rows, int nz, const float *angles,
                         const float *zs, const double *proj, double *vol, int batch,
                         int transpose) {
    const int V = g->n_views, C = g->n_cols, nx = g->nx, ny = g->ny;
    const double r2 = (double)g->rfov * (double)g->rfov;
    const float zmin = -0.5f * g->dz * (float)nz;
    const size_t pview = (size_t)n_rows * C, pvol = (size_t)nz * ny * nx;
    if (transpose) memset((void *)proj, 0, sizeof(double) * batch * V * pview);
    for (int b = 0; b < batch; ++b) {
        const double *pb = proj + (size_t)b * V * pview;
        double *vb = vol + (size_t)b * pvol;
        if (!transpose) {
#pragma omp parallel for schedule(dynamic, 2)
            for (int j = 0; j < ny; ++j) {
                const double y = (double)g->ymin + (double)g->dy * (j + 0.5);
                for (int i = 0; i < nx; ++i) {
                    const double x = (double)g->xmin + (double)g->dx * (i + 0.5);
                    for (int k = 0; k < nz; ++k) vb[((size_t)k * ny + j) * nx + i] = 0.0;
                    if (!(x * x + y * y <= r2)) continue;
                    for (int v = 0; v < V; ++v) {
                        const double beta = angles[v];
                        const double c = -cos(beta), s = -sin(beta);
                        int i0, i1;
                        double f, U, t;
                        if (!bp_col(g, x, y, c, s, &i0, &i1, &f, &U, &t)) continue;
                        const double wgt = 1.0 / (U * U + t * t);
                        const double *pv = pb + (size_t)v * pview;
                        const double z_src = zs ? (double)zs[v] : 0.0;
                        for (int k = 0; k < nz; ++k) {
                            const double zk = (double)zmin + (double)g->dz * (k + 0.5) - z_src;
                            const double row =
                                (zk * (double)g->sdd / U - (double)g->det_bottom) / (double)g->drow;
                            const double rb = row - 0.5, rf = floor(rb);
                            const double fr = frac_w(rb - rf);
                            const int q = (int)rf;
                            const int ra = q < 0 ? 0 : (q > n_rows - 1 ? n_rows - 1 : q);
                            const int rc = q + 1 < 0 ? 0 : (q + 1 > n_rows - 1 ? n_rows - 1 : q + 1);
                            const double *va = pv + (size_t)ra * C, *vc = pv + (size_t)rc * C;
                            double w[4];
                            bilinear_w(f, fr, w);
                            vb[((size_t)k * ny + j) * nx + i] +=
                                (w[0] * va[i0] + w[1] * va[i1] + w[2] * vc[i0] + w[3] * vc[i1]) *
                                wgt;
                        }
                    }
                }
            }
        } else {
            double *pw = (double *)(proj + (size_t)b * V * pview);
#pragma omp parallel for schedule(dynamic, 2)
            for (int v = 0; v < V; ++v) {
                const double beta = angles[v];
                const double c = -cos(beta), s = -sin(beta);
                double *pv = pw + (size_t)v * pview;
                for (int j = 0; j < ny; ++j) {
                    const double y = (double)g->ymin + (double)g->dy * (j + 0.5);
                    for (int i = 0; i < nx; ++i) {
                        const double x = (double)g->xmin + (double)g->dx * (i + 0.5);
                        int i0, i1;
                        double f, U, t;
                        if (!(x * x + y * y <= r2)) continue;
                        if (!bp_col(g, x, y, c, s, &i0, &i1, &f, &U, &t)) continue;
                        const double wgt = 1.0 / (U * U + t * t);
                        const double z_src = zs ? (double)zs[v] : 0.0;
                        for (int k = 0; k < nz; ++k) {
                            const double val = vb[((size_t)k * ny + j) * nx + i] * wgt;
                            const double zk = (double)zmin + (double)g->dz * (k + 0.5) - z_src;
                            const double row =
                                (zk * (double)g->sdd / U - (double)g->det_bottom) / (double)g->drow;
                            const double rb = row - 0.5, rf = floor(rb);
                            const double fr = frac_w(rb - rf);
                            const int q = (int)rf;
                            const int ra = q < 0 ? 0 : (q > n_rows - 1 ? n_rows - 1 : q);
                            const int rc = q + 1 < 0 ? 0 : (q + 1 > n_rows - 1 ? n_rows - 1 : q + 1);
                            if (val == 0.0) continue;
                            double w[4];
                            bilinear_w(f, fr, w);
                            pv[(size_t)ra * C + i0] += val * w[0];
                            pv[(size_t)ra * C + i1] += val * w[1];
                            pv[(size_t)rc * C + i0] += val * w[2];
                            pv[(size_t)rc * C + i1] += val * w[3];
                        }
                    }
                }
            }
        }
    }
}

void orc_cone_bp(const orc_geom *g, int n_rows, int nz, const float *angles, const double *proj,
                 double *vol, int batch) {
    cone_bp_impl(g, n_rows, nz, angles, NULL, proj, vol, batch, 0);
}

void orc_cone_bp_transpose(const orc_geom *g, int n_rows, int nz, const float *angles,
                           const double *vol, double *proj, int batch) {
    cone_bp_impl(g, n_rows, nz, angles, NULL, proj, (double *)vol, batch, 1);
}

/* The same with the source of view v at height zs[v] (mm): the row of a voxel
 * at z is ((z - zs[v]) * D / U - det_bottom) / drow. */
void orc_cone_bp_zs(const orc_geom *g, int n_rows, int nz, const float *angles, const float *zs,
                    const double *proj, double *vol, int batch) {
    cone_bp_impl(g, n_rows, nz, angles, zs, proj, vol, batch, 0);
}

void orc_cone_bp_transpose_zs(const orc_geom *g, int n_rows, int nz, const float *angles,
                              const float *zs, const double *vol, double *proj, int batch) {
    cone_bp_impl(g, n_rows, nz, angles, zs, proj, (double *)vol, batch, 1);
}

/* FDK of the reference (BP_One_Rot_3D_GPU, FDK/GPURecon_GPU.cu:163-268) with
 * nz slices and n_rows detector rows: ramp filter every (view, row), then the
 * CB_EA backprojection.  orc_fdk_bp is its nz = n_rows = 1 case. */
void orc_fdk_cone(const orc_geom *g, int n_rows, int nz, const float *angles, int window,
                  const double *proj, double *vol, int batch) {
    const size_t n = (size_t)batch * g->n_views * n_rows * g->n_cols;
    double *filt = (double *)malloc(sizeof(double) * (n ? n : 1));
    orc_ramp_filter(g, window, proj, filt, (long)batch * g->n_views * n_rows);
    orc_cone_bp(g, n_rows, nz, angles, filt, vol, batch);
    free(filt);
}

/* Transpose of orc_fdk_cone: CB_EA transpose, then the symmetric filter. */
void orc_fdk_cone_adjoint(const orc_geom *g, int n_rows, int nz, const float *angles, int window,
                          const double *vol, double *proj, int batch) {
    const size_t n = (size_t)batch * g->n_views * n_rows * g->n_cols;
    double *tmp = (double *)malloc(sizeof(double) * (n ? n : 1));
    orc_cone_bp_transpose(g, n_rows, nz, angles, vol, tmp, batch);
    orc_ramp_filter(g, window, tmp, proj, (long)batch * g->n_views * n_rows);
    free(tmp);
}

/* Cone-beam forward projection (no reference counterpart: the reference
 * removed its cone projector and kept only unused 3-D textures,
 * FDK/GPURecon_GPU.cu:10,12).  Detector cell (view v, row r, channel i) is
 * the point at height h_r = det_bottom + (r+1/2) drow on the cylinder of
 * radius D about the source, at fan angle left + (i+1/2) dcol.  The ray from
 * the source to it is sampled at the in-plane positions of the fan-beam
 * projector (start + k*step, k < n, orc_ray_table); at in-plane distance s
 * from the source the ray's height is z = h_r * s / D.  Each sample is a
 * trilinear, clamp-to-edge volume sample (texel centres at +1/2 in x, y, z),
 * and the sum is weighted by 0.125*dx*sqrt(1 + (h_r/D)^2), the 3-D length of
 * one in-plane step. */
static void cone_fp_impl(const orc_geom *g, int n_rows, int nz, const float *angles,
                         const float *zs, const double *vol, double *proj, int batch) {
    const int V = g->n_views, C = g->n_cols, nx = g->nx, ny = g->ny;
    const size_t R = (size_t)V * C;
    double *ray = (double *)malloc(sizeof(double) * 4 * R);
    int32_t *ns = (int32_t *)malloc(sizeof(int32_t) * R);
    const double dx = g->dx, D = g->sdd;
    const double src = (double)g->sid / dx, fov = (double)g->rfov / dx;
    const float zmin = -0.5f * g->dz * (float)nz;
    const size_t pvol = (size_t)nz * ny * nx;
    orc_ray_table(g, angles, ray, ns);
    for (int b = 0; b < batch; ++b) {
        const double *vb = vol + (size_t)b * pvol;
        double *pb = proj + (size_t)b * V * n_rows * C;
#pragma omp parallel for schedule(dynamic, 16)
        for (long rr = 0; rr < (long)R; ++rr) {
            const int v = (int)(rr / C), i = (int)(rr % C);
            const double *q = ray + 4 * rr;
            const int n = ns[rr];
            /* in-plane distance (mm) from the source of sample k: s0 + k*ds */
            const double gam = (double)g->left + (i + 0.5) * (double)g->dcol;
            const double dist = src * sin(gam);
            const double h = fov * fov - dist * dist;
            double s0 = 0.0, ds = 0.0;
            if (n > 0) {
                const double x1 = -sqrt(h);
                const double L = 2.0 * sqrt(h);
                s0 = dx * (src * cos(gam) - x1);
                ds = -dx * L / n;
            }
            for (int r = 0; r < n_rows; ++r) {
                const double hr = (double)g->det_bottom + (r + 0.5) * (double)g->drow;
                double acc = 0.0;
                for (int k = 0; k < n; ++k) {
                    const tap4 t = bilinear_taps(nx, ny, q[0] + k * q[2], q[1] + k * q[3]);
                    const double z = (zs ? (double)zs[v] : 0.0) + hr * (s0 + k * ds) / D;
                    const double wz = (z - (double)zmin) / (double)g->dz - 0.5;
                    const double fz0 = floor(wz);
                    const double az = frac_w(wz - fz0);
                    const int kz = (int)fz0;
                    const int k0 = kz < 0 ? 0 : (kz > nz - 1 ? nz - 1 : kz);
                    const int k1 = kz + 1 < 0 ? 0 : (kz + 1 > nz - 1 ? nz - 1 : kz + 1);
                    const double *p0 = vb + (size_t)k0 * ny * nx, *p1 = vb + (size_t)k1 * ny * nx;
                    const double a0 = t.w00 * p0[t.j0 * nx + t.i0] + t.w10 * p0[t.j0 * nx + t.i1] +
                                      t.w01 * p0[t.j1 * nx + t.i0] + t.w11 * p0[t.j1 * nx + t.i1];
                    const double a1 = t.w00 * p1[t.j0 * nx + t.i0] + t.w10 * p1[t.j0 * nx + t.i1] +
                                      t.w01 * p1[t.j1 * nx + t.i0] + t.w11 * p1[t.j1 * nx + t.i1];
                    acc += (1.0 - az) * a0 + az * a1;
                }
                pb[((size_t)v * n_rows + r) * C + i] =
                    acc * ORC_STEP * dx * sqrt(1.0 + (hr / D) * (hr / D));
            }
        }
    }
    free(ray);
    free(ns);
}

void orc_cone_fp(const orc_geom *g, int n_rows, int nz, const float *angles, const double *vol,
                 double *proj, int batch) {
    cone_fp_impl(g, n_rows, nz, angles, NULL, vol, proj, batch);
}

/* Cone FP with the source of view v at height zs[v]: the ray's height at
 * in-plane distance s is zs[v] + h_r * s / D. */
void orc_cone_fp_zs(const orc_geom *g, int n_rows, int nz, const float *angles, const float *zs,
                    const double *vol, double *proj, int batch) {
    cone_fp_impl(g, n_rows, nz, angles, zs, vol, proj, batch);
}

/* Feldkamp cosine pre-weights [n_rows][C]: cos(gam_i), times
 * D / sqrt(D^2 + h_r^2) when cone != 0 (the cone angle of row r of the
 * cylindrical detector), gam_i = left + (i + 1/2 - shift) dcol. */
void orc_cosine_weights(const orc_geom *g, int n_rows, int cone, double *w) {
    const int C = g->n_cols;
    const double D = g->sdd;
    for (int r = 0; r < n_rows; ++r) {
        const double h = (double)g->det_bottom + (r + 0.5) * (double)g->drow;
        for (int i = 0; i < C; ++i) {
            const double gam = (double)g->left + (i + 0.5 - (double)g->shift) * (double)g->dcol;
            /* cos(gam) * cos(kappa) with tan(kappa) = h / D */
            const double ck = cone ? 1.0 / sqrt(1.0 + (h / D) * (h / D)) : 1.0;
            w[(size_t)r * C + i] = cos(gam) * ck;
        }
    }
}
