// Host-side geometry: parameter decoding and the FP64-derived per-view and
// per-ray tables the kernels consume.  Built with -ffp-contract=off so the
// double-precision tables are identical on x86-64 and aarch64 hosts.
#include <cmath>
#include <cstring>
#include <utility>

#include "internal.h"

namespace {
bool finite(float v) { return std::isfinite(v); }
// Truncation toward zero of a float attribute, as int(parameter(k)) does in
// the reference constructors (FP/transform.cc:61,64-66,75).
bool to_int(float v, int32_t *out) {
    if (!finite(v) || v <= -2147483648.0f || v >= 2147483648.0f) return false;
    *out = static_cast<int32_t>(v);
    return true;
}
}  // namespace

// Mirrors FPFanCurveOp's constructor arithmetic (FP/transform.cc:59-76) and the
// FDK op's extra fields (FDK/FBP.cc:82-84), in float, term for term.
ct_status ct_decode_param16(const float p[16], ct_fan_geom *g) {
    if (!p || !g) return CT_ERR_NULL_POINTER;
    std::memset(g, 0, sizeof(*g));
    const float PI = CT_REF_PI;
    g->sdd = p[0];
    g->sid = p[1];
    if (!to_int(p[2], &g->n_views)) return CT_ERR_INVALID_ARGUMENT;
    g->full_angle = p[3];
    if (!to_int(p[4], &g->n_cols)) return CT_ERR_INVALID_ARGUMENT;
    if (!to_int(p[5], &g->nx)) return CT_ERR_INVALID_ARGUMENT;
    if (!to_int(p[6], &g->ny)) return CT_ERR_INVALID_ARGUMENT;
    g->rfov = p[7];
    g->shift = p[9];
    if (!to_int(p[11], &g->n_slices)) return CT_ERR_INVALID_ARGUMENT;
    g->det_bottom = p[13];
    g->drow = p[14];
    g->dz = p[15];
    if (g->n_views <= 0 || g->nx <= 0 || g->ny <= 0) return CT_ERR_INVALID_ARGUMENT;
    // dAngle = dRange/nViews*PI/180.0f (FP/transform.cc:63)
    float d_angle = g->full_angle / static_cast<float>(g->n_views);
    d_angle = d_angle * PI;
    g->d_angle = d_angle / 180.0f;
    // dx = 2.0f*rFOV/nX; xmin = -0.5f*nX*dx (FP/transform.cc:68-71)
    float two_r = 2.0f * g->rfov;
    g->dx = two_r / static_cast<float>(g->nx);
    g->dy = two_r / static_cast<float>(g->ny);
    float hx = -0.5f * static_cast<float>(g->nx);
    float hy = -0.5f * static_cast<float>(g->ny);
    g->xmin = hx * g->dx;
    g->ymin = hy * g->dy;
    // dCol, dLeft, start angle: parameter(k)*PI/180.0f (FP/transform.cc:72-76)
    float t = p[8] * PI;
    g->dcol = t / 180.0f;
    t = p[10] * PI;
    g->left = t / 180.0f;
    t = p[12] * PI;
    g->start_angle = t / 180.0f;
    return ct_validate_geom(g);
}

// The reference checks nothing; these are the conditions under which its
// formulas describe a real fan-beam scan (pixels in front of the source, a
// non-degenerate detector) and under which 32-bit indexing is safe.
ct_status ct_validate_geom(const ct_fan_geom *g) {
    if (!g) return CT_ERR_NULL_POINTER;
    if (g->n_views <= 0 || g->n_cols <= 0 || g->nx <= 0 || g->ny <= 0)
        return CT_ERR_INVALID_ARGUMENT;
    if ((int64_t)g->n_views * g->n_cols >= (int64_t)1 << 31) return CT_ERR_INVALID_ARGUMENT;
    if ((int64_t)g->nx * g->ny >= (int64_t)1 << 31) return CT_ERR_INVALID_ARGUMENT;
    if (g->nx > 32768 || g->ny > 32768 || g->n_cols > (1 << 20)) return CT_ERR_INVALID_ARGUMENT;
    const float vals[] = {g->sdd, g->sid, g->full_angle, g->rfov, g->shift, g->det_bottom,
                          g->drow,  g->dz,  g->d_angle,    g->dx,   g->dy,    g->xmin,
                          g->ymin,  g->dcol, g->left};
    for (float v : vals)
        if (!finite(v)) return CT_ERR_INVALID_ARGUMENT;
    if (!(g->rfov > 0.0f) || !(g->sid > g->rfov)) return CT_ERR_INVALID_ARGUMENT;
    if (!(g->dcol > 0.0f) || !(g->dx > 0.0f) || !(g->dy > 0.0f)) return CT_ERR_INVALID_ARGUMENT;
    return CT_OK;
}

// c = -cos(beta), s = -sin(beta): the reference passes -sinf(angle) and
// -cosf(angle) to every BP kernel (BP/transform.cu:116, FBP/transform.cu:110,
// FDK/GPURecon_GPU.cu:255).
void ct_build_view_table(const ct_fan_geom *g, const float *angles, ct_host_tables *t) {
    const int V = g->n_views;
    t->view_cs.assign(2 * (size_t)V, 0.0f);
    t->view_cs_lo.assign(2 * (size_t)V, 0.0f);
    for (int v = 0; v < V; ++v) {
        const double beta = angles[v];
        const double c = -std::cos(beta), s = -std::sin(beta);
        t->view_cs[2 * v + 0] = static_cast<float>(c);
        t->view_cs[2 * v + 1] = static_cast<float>(s);
        t->view_cs_lo[2 * v + 0] = static_cast<float>(c - (double)t->view_cs[2 * v + 0]);
        t->view_cs_lo[2 * v + 1] = static_cast<float>(s - (double)t->view_cs[2 * v + 1]);
    }
    // column boundaries y = b: gamma_b = left + (b - shift - 1/2) dcol, the
    // inverse of y = (gamma - left)/dcol + shift + 1/2 (BP/transform.cu:86)
    const int C = g->n_cols;
    t->col_tan.assign(2 * (size_t)(C + 1), 0.0f);
    for (int b = 0; b <= C; ++b) {
        const double tg =
            std::tan((double)g->left + ((double)b - (double)g->shift - 0.5) * (double)g->dcol);
        const float hi = static_cast<float>(tg);
        t->col_tan[2 * (size_t)b] = hi;
        t->col_tan[2 * (size_t)b + 1] = static_cast<float>(tg - (double)hi);
    }
}

// Per-ray table of GenerateRayTraceMap_FB_ReconImage_OneView_kernel
// (FP/transform.cu:64-101), evaluated in double: ray angle
// beta + left + (i+1/2) dcol, signed distance R/dx * sin(gamma) of the ray from
// the isocentre, the two intersections of the ray with the FOV circle of
// radius rfov/dx (pixel units), chord length L, n = floor(L/0.125), start =
// first intersection + rfov/dx, step = chord/n.  A ray that misses the circle
// (the reference's sqrtf of a negative number, :81) or touches it (L = 0)
// gets n = 0 and contributes 0.
void ct_build_ray_table(const ct_fan_geom *g, const float *angles, ct_host_tables *t) {
    const int V = g->n_views, C = g->n_cols;
    const size_t R = (size_t)V * C;
    t->ray.assign(4 * R, 0.0f);
    t->nsamp.assign(R, 0);
    t->max_nsamp = 0;
    t->total_samples = 0;
    const double dx = g->dx;
    const double src_px = (double)g->sid / dx;
    const double fov_px = (double)g->rfov / dx;
    const double left = g->left, dcol = g->dcol;
    for (int v = 0; v < V; ++v) {
        const double beta = angles[v];
        for (int i = 0; i < C; ++i) {
            const size_t r = (size_t)v * C + i;
            const double gam = left + (i + 0.5) * dcol;
            const double th = beta + gam;
            const double sn = std::sin(th), cs = std::cos(th);
            const double dist = src_px * std::sin(gam);
            const double h = fov_px * fov_px - dist * dist;
            if (!(h > 0.0)) continue;
            const double x1 = -std::sqrt(h), x2 = -x1, y1 = -dist, y2 = -dist;
            const double ax = x1 * cs - y1 * sn, ay = x1 * sn + y1 * cs;
            const double bx = x2 * cs - y2 * sn, by = x2 * sn + y2 * cs;
            const double L = std::sqrt((ax - bx) * (ax - bx) + (ay - by) * (ay - by));
            const double q = std::floor(L / CT_FP_STEP);
            if (!(q >= 1.0)) continue;
            const int32_t n = static_cast<int32_t>(q);
            t->nsamp[r] = n;
            t->ray[4 * r + 0] = static_cast<float>(ax + fov_px);
            t->ray[4 * r + 1] = static_cast<float>(ay + fov_px);
            t->ray[4 * r + 2] = static_cast<float>((bx - ax) / n);
            t->ray[4 * r + 3] = static_cast<float>((by - ay) / n);
            if (n > t->max_nsamp) t->max_nsamp = n;
            t->total_samples += n;
        }
    }
}

// Ramp filter taps h[n], n in [-(C-1), C-1], stored at index n + C - 1 and
// multiplied by R * d_angle * dcol (FBP/transform.cu:149-162,
// FDK/GPURecon_GPU.cu:184-200).  Ram-Lak is Hsieh's equiangular h'' form with
// the 0.5 redundancy factor: h[0] = 0.5/(4 dcol^2), h[odd n] =
// -0.5/(pi^2 sin^2(n dcol)), h[even n != 0] = 0.  Shepp-Logan is
// 0.5 * 2/(pi^2 dcol^2 (1-4n^2)) mapped to the fan by (n dcol/sin(n dcol))^2.
void ct_build_filter_taps(const ct_fan_geom *g, int window, ct_host_tables *t) {
    const int C = g->n_cols;
    t->taps.assign(2 * (size_t)C - 1, 0.0f);
    const double pi = (double)CT_REF_PI;
    const double dc = g->dcol;
    const double scale = (double)g->sid * (double)g->d_angle * dc;
    for (int n = -(C - 1); n <= C - 1; ++n) {
        double h;
        if (window == CT_WINDOW_SHEPP_LOGAN) {
            if (n == 0) {
                h = 0.5 * 2.0 / (pi * pi * dc * dc);
            } else {
                const double s = std::sin(n * dc);
                h = 0.5 * 2.0 * (double)n * (double)n /
                    (pi * pi * s * s * (1.0 - 4.0 * (double)n * (double)n));
            }
        } else {
            if (n == 0) {
                h = 0.5 / (4.0 * dc * dc);
            } else if (n % 2 != 0) {
                const double s = std::sin(n * dc);
                h = -0.5 / (pi * pi * s * s);
            } else {
                h = 0.0;
            }
        }
        t->taps[(size_t)(n + C - 1)] = static_cast<float>(h * scale);
    }
}

double ct_max_tan_gamma(const ct_fan_geom *g) {
    const double r = g->rfov, R = g->sid;
    return r / std::sqrt(R * R - r * r);
}

namespace {
// Solves the (n x n, n <= 9) system A x = b by Gaussian elimination with
// partial pivoting; A is row-major and overwritten.
void solve_small(double *A, double *b, int n) {
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(A[r * n + c]) > std::fabs(A[piv * n + c])) piv = r;
        if (piv != c) {
            for (int k = 0; k < n; ++k) std::swap(A[c * n + k], A[piv * n + k]);
            std::swap(b[c], b[piv]);
        }
        for (int r = c + 1; r < n; ++r) {
            const double f = A[r * n + c] / A[c * n + c];
            for (int k = c; k < n; ++k) A[r * n + k] -= f * A[c * n + k];
            b[r] -= f * b[c];
        }
    }
    for (int c = n - 1; c >= 0; --c) {
        double s = b[c];
        for (int k = c + 1; k < n; ++k) s -= A[c * n + k] * b[k];
        b[c] = s / A[c * n + c];
    }
}
}  // namespace

// atan(z)/z is smooth and even, so it is interpolated as a polynomial in
// s = z^2 on [0, zmax^2] at the deg+1 Chebyshev nodes (solved in the scaled
// variable x = s/zmax^2 for conditioning), then checked on a dense grid.
int ct_fit_atan(double zmax, float coef[9]) {
    const double pi = 3.14159265358979323846;
    for (int k = 0; k < 9; ++k) coef[k] = 0.0f;
    if (!(zmax > 0.0) || zmax > 1.0) return 0;
    const double smax = zmax * zmax;
    const int degs[2] = {4, 8};
    for (int deg : degs) {
        const int n = deg + 1;
        double A[81], b[9];
        for (int i = 0; i < n; ++i) {
            const double x = 0.5 * (1.0 - std::cos((2.0 * i + 1.0) * pi / (2.0 * n)));
            const double s = x * smax, z = std::sqrt(s);
            b[i] = s > 0.0 ? std::atan(z) / z : 1.0;
            double xp = 1.0;
            for (int k = 0; k < n; ++k) {
                A[i * n + k] = xp;
                xp *= x;
            }
        }
        solve_small(A, b, n);
        double c[9];
        double scale = 1.0;
        for (int k = 0; k < n; ++k) {
            c[k] = b[k] / scale;  // coefficient of s^k
            scale *= smax;
        }
        double err = 0.0;
        for (int i = 0; i <= 4000; ++i) {
            const double z = zmax * i / 4000.0, s = z * z;
            double p = c[deg];
            for (int k = deg - 1; k >= 0; --k) p = p * s + c[k];
            err = std::fmax(err, std::fabs(z * p - std::atan(z)));
        }
        if (err <= 3e-8) {
            for (int k = 0; k < n; ++k) coef[k] = static_cast<float>(c[k]);
            return deg;
        }
    }
    return 0;
}

// In-plane geometry of the cone-beam projector's rays, per channel i (the
// same for every view): with gamma = left + (i+1/2) dcol, the ray's distance
// from the isocentre is d = R sin(gamma), its FOV chord 2 sqrt(rfov^2 - d^2),
// and its first sample (the far chord end) lies R cos(gamma) + sqrt(rfov^2 -
// d^2) from the source; both in mm, evaluated in pixel units as the ray table.
void ct_build_channel_table(const ct_fan_geom *g, ct_host_tables *t) {
    const int C = g->n_cols;
    t->chan_s.assign(2 * (size_t)C, 0.0f);
    const double dx = g->dx;
    const double src_px = (double)g->sid / dx, fov_px = (double)g->rfov / dx;
    for (int i = 0; i < C; ++i) {
        const double gam = (double)g->left + (i + 0.5) * (double)g->dcol;
        const double dist = src_px * std::sin(gam);
        const double h = fov_px * fov_px - dist * dist;
        if (!(h > 0.0)) continue;
        const double x1 = -std::sqrt(h);
        t->chan_s[2 * i + 0] = static_cast<float>(dx * (src_px * std::cos(gam) - x1));
        t->chan_s[2 * i + 1] = static_cast<float>(dx * 2.0 * std::sqrt(h));
    }
}

// Feldkamp cosine pre-weights (L. A. Feldkamp, L. C. Davis, J. W. Kress,
// JOSA A 1(6), 1984) per (row, channel) of an equiangular, cylindrical
// detector: cos(gamma_i), times the cosine of the row's cone angle,
// D / sqrt(D^2 + h_r^2) with h_r = det_bottom + (r + 1/2) drow, for cone
// plans; gamma_i = left + (i + 1/2 - shift) dcol as the backprojector maps it.
void ct_build_cosine(const ct_fan_geom *g, int n_rows, bool cone, ct_host_tables *t) {
    const int C = g->n_cols;
    const double D = g->sdd;
    t->cosw.assign((size_t)n_rows * C, 0.0f);
    for (int r = 0; r < n_rows; ++r) {
        const double h = (double)g->det_bottom + (r + 0.5) * (double)g->drow;
        const double kappa = cone ? D / std::sqrt(D * D + h * h) : 1.0;
        for (int i = 0; i < C; ++i) {
            const double gam = (double)g->left + (i + 0.5 - (double)g->shift) * (double)g->dcol;
            t->cosw[(size_t)r * C + i] = static_cast<float>(std::cos(gam) * kappa);
        }
    }
}

// Parker's short-scan weights (D. L. Parker, Med. Phys. 9(2), 1982) for the
// ray of view v and channel i: with beta = angle[v] - angle[0] and the
// channel's fan angle gamma = left + (i + 1/2 - shift) dcol (the angle the
// backprojector assigns to that channel), and Gamma the half fan angle (the
// outer edge of the outermost channel),
//   w = sin^2(pi/4 beta/(Gamma - gamma))            0 <= beta < 2(Gamma - gamma)
//     = 1                                           ... < pi - 2 gamma
//     = sin^2(pi/4 (pi + 2 Gamma - beta)/(Gamma + gamma))  ... <= pi + 2 Gamma
//     = 0                                           otherwise.
// In this geometry the same line is measured again at (beta + pi + 2 gamma,
// -gamma), and the two weights sum to one.  A scan whose angles decrease is
// the mirror image: beta and gamma change sign.  Stored doubled, because the
// ramp taps carry the 0.5 of full-scan redundancy (FBP/transform.cu:156-158).
void ct_build_parker(const ct_fan_geom *g, const float *angles, ct_host_tables *t) {
    const int V = g->n_views, C = g->n_cols;
    const double pi = 3.14159265358979323846;
    const double dcol = g->dcol;
    const double dir = (V > 1 && angles[V - 1] < angles[0]) ? -1.0 : 1.0;
    const double g0 = (double)g->left + (0.5 - (double)g->shift) * dcol;
    const double g1 = (double)g->left + (C - 0.5 - (double)g->shift) * dcol;
    const double G = std::fmax(std::fabs(g0), std::fabs(g1)) + 0.5 * dcol;
    t->parker.assign((size_t)V * C, 0.0f);
    for (int v = 0; v < V; ++v) {
        const double beta = dir * ((double)angles[v] - (double)angles[0]);
        for (int i = 0; i < C; ++i) {
            const double gam = dir * ((double)g->left + (i + 0.5 - (double)g->shift) * dcol);
            double w = 0.0;
            if (beta >= 0.0 && beta < 2.0 * (G - gam)) {
                const double s = std::sin(pi / 4.0 * beta / (G - gam));
                w = s * s;
            } else if (beta >= 2.0 * (G - gam) && beta < pi - 2.0 * gam) {
                w = 1.0;
            } else if (beta >= pi - 2.0 * gam && beta <= pi + 2.0 * G) {
                const double s = std::sin(pi / 4.0 * (pi + 2.0 * G - beta) / (G + gam));
                w = s * s;
            }
            t->parker[(size_t)v * C + i] = static_cast<float>(2.0 * w);
        }
    }
}

// Tables of the gather-form BP transpose (bp_gather.cu).  For view v the
// detector columns are cut into strips between boundary rays: strip b holds
// the pixels whose column coordinate y = col + 1/2 lies in [b, b+1) -- the
// pixels whose two clamped taps are (max(b-1, 0), min(b, C-1)) -- with the
// outer strips cut at y = 1/2 and y = C + 1/2, where the backprojector's test
// 0 < col < C ends (BP/transform.cu:88).  Boundary y = B lies on the ray
// from the source at fan angle gamma = left + (B - shift - 1/2) dcol.  A warp
// takes 32 consecutive strips (31 new per warp, channel group k: strips
// 31k .. 31k+31) and walks the image lines across its rays: rows when the
// rays run more along y, columns otherwise.  Per line the strip's pixels
// lie between the two boundary rays' crossings of the line, and per pixel
// the fraction f = (gamma_p - gamma_b)/dcol follows from the pixel's offset
// from the lower boundary's crossing (exact, in 32.32 fixed point along the
// line), never from the absolute column coordinate, whose FP32 rounding the
// ramp filter of the FBP adjoint would amplify.
void ct_build_bpt_tables(const ct_fan_geom *g, const float *angles, ct_bpt_tables *t) {
    const int V = g->n_views, C = g->n_cols;
    const int W = (C + kBptOut - 1) / kBptOut;
    t->W = W;
    t->ok = true;
    t->warp.assign((size_t)V * W * 4, 0);
    t->bnd.assign((size_t)V * W * 33 * 2, 0);
    t->ray.assign((size_t)V * W * 32 * 4, 0.0f);
    const double R = g->sid, dcol = g->dcol, left = g->left, shift = g->shift;
    const double dx = g->dx, dy = g->dy, xmin = g->xmin, ymin = g->ymin;
    const double r2 = (double)g->rfov * (double)g->rfov;
    // per line, the inclusive pixel range inside the FOV disc (the
    // backprojectors' own double-precision test)
    t->fov_row.assign((size_t)g->ny * 2, 0);
    t->fov_col.assign((size_t)g->nx * 2, 0);
    for (int pass = 0; pass < 2; ++pass) {
        const int nl = pass ? g->nx : g->ny, np = pass ? g->ny : g->nx;
        std::vector<int32_t> &f = pass ? t->fov_col : t->fov_row;
        for (int l = 0; l < nl; ++l) {
            int lo = np, hi = -1;
            for (int q = 0; q < np; ++q) {
                const int ix = pass ? l : q, iy = pass ? q : l;
                const double xd = xmin + dx * (ix + 0.5), yd = ymin + dy * (iy + 0.5);
                if (xd * xd + yd * yd <= r2) {
                    lo = q < lo ? q : lo;
                    hi = q;
                }
            }
            f[2 * (size_t)l] = lo;
            f[2 * (size_t)l + 1] = hi;
        }
    }
    const double rlim = (double)g->rfov + 2.0 * (dx > dy ? dx : dy);
    const double two32 = 4294967296.0;
    for (int v = 0; v < V; ++v) {
        const double beta = (double)angles[v];
        const double c = -std::cos(beta), s = -std::sin(beta);
        const double Sx = -R * c, Sy = -R * s;  // the source; e_u = (c, s), e_t = (-s, c)
        for (int k = 0; k < W; ++k) {
            double d[33][2], n[33][2];
            int along_y = 0, valid = 0;
            for (int q = 0; q < 33; ++q) {
                const int b = k * kBptOut + q;
                const double B = b <= 0 ? 0.5 : (b >= C + 1 ? C + 0.5 : (double)b);
                const double gam = left + (B - shift - 0.5) * dcol;
                const double cg = std::cos(gam), sg = std::sin(gam);
                d[q][0] = cg * c - sg * s;
                d[q][1] = cg * s + sg * c;
                n[q][0] = -sg * c - cg * s;
                n[q][1] = -sg * s + cg * c;
                if (b <= C + 1) {
                    ++valid;
                    along_y += std::fabs(d[q][1]) >= std::fabs(d[q][0]);
                }
            }
            const int layout = 2 * along_y >= valid ? 0 : 1;  // 0: walk rows, 1: walk columns
            const int aw = layout ? 0 : 1, ap = 1 - aw;         // walk / pixel axis components
            const double lmin = layout ? xmin : ymin, dl = layout ? dx : dy;
            const double pmin = layout ? ymin : xmin, dp = layout ? dy : dx;
            const double Sw = layout ? Sx : Sy, Sp = layout ? Sy : Sx;
            const int nlines = layout ? g->nx : g->ny;
            int orient = 0;
            double jmin = 1e300, jmax = -1e300;
            for (int q = 0; q < 33; ++q) {
                if (k * kBptOut + q > C + 1) break;
                if (std::fabs(d[q][aw]) < 0.2) t->ok = false;
                const int o = n[q][ap] > 0.0 ? 1 : -1;
                if (orient && o != orient) t->ok = false;
                orient = o;
                // the ray's chord of the FOV disc (widened), in line indices
                const double dist = std::fabs(Sx * d[q][1] - Sy * d[q][0]);
                if (dist < rlim) {
                    const double lm = -(Sx * d[q][0] + Sy * d[q][1]);
                    const double h = std::sqrt(rlim * rlim - dist * dist);
                    for (double L : {lm - h, lm + h}) {
                        const double w = Sw + L * d[q][aw];
                        const double jl = (w - lmin) / dl - 0.5;
                        jmin = jl < jmin ? jl : jmin;
                        jmax = jl > jmax ? jl : jmax;
                    }
                }
            }
            int J0 = 1, J1 = 0;
            if (jmax >= jmin) {
                J0 = (int)std::floor(jmin) - 2;
                J1 = (int)std::ceil(jmax) + 2;
                J0 = J0 < 0 ? 0 : J0;
                J1 = J1 > nlines - 1 ? nlines - 1 : J1;
            }
            const size_t e = (size_t)v * W + k;
            t->warp[4 * e] = layout | (orient > 0 ? 2 : 0);
            t->warp[4 * e + 1] = J0;
            t->warp[4 * e + 2] = J1;
            const double wl = lmin + dl * (J0 + 0.5);  // line J0's coordinate
            for (int q = 0; q < 33; ++q) {
                const double dw = std::fabs(d[q][aw]) < 1e-12 ? 1e-12 : d[q][aw];
                const double L0 = (wl - Sw) / dw;  // along the ray to line J0
                const double X0 = (Sp + L0 * d[q][ap] - pmin) / dp - 0.5;
                const double step = dl / dw * d[q][ap] / dp;
                const double lim = 4.0e9;  // far beyond any image: clamp, the range is then empty
                auto fx = [&](double x) {
                    x = x > lim ? lim : (x < -lim ? -lim : x);
                    return (int64_t)std::llround(x * two32);
                };
                t->bnd[2 * (e * 33 + q)] = fx(X0);
                t->bnd[2 * (e * 33 + q) + 1] = fx(step);
                if (q < 32) {
                    float *r = &t->ray[4 * (e * 32 + q)];
                    r[0] = (float)L0;
                    r[1] = (float)(dl / dw);
                    r[2] = (float)(dp * n[q][ap]);
                    r[3] = (float)(dp * d[q][ap]);
                }
            }
        }
    }
}
