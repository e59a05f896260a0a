/*
 * CPU oracle for the live-dic IC-GN hot path.  TEST INFRASTRUCTURE ONLY:
 * the product library never links, loads or calls this file.  It is used by
 * tests/, by __graft_entry__.smoke() as the checker, and by bench.py's CPU
 * baseline leg.
 *
 * It restates, in plain C, the WGSL kernels of the reference
 * (DIC/LucasKanadeICGN/python/src/live_dic/shaders/):
 *   - icgn.wgsl:128-214   mirrored 25-tap FIR target prefilter (x then y)
 *   - icgn.wgsl:230-319   cubic B-spline / bilinear / Keys interpolants
 *   - icgn.wgsl:321-593   increments, inverse composition, change, status
 *   - icgn.wgsl:595-1017  solve_subset and its zero-seed / seeded / retry entries
 *   - icgn.wgsl:1087-1605 UOD (flag/replace) and median repair
 *   - full_pyramid.wgsl:150-249 exact integer 5x5 pyramid reduction
 *   - full_pyramid.wgsl:251-435 coarse-to-fine seed transfer
 *   - full_pyramid.wgsl:83-148,437-575 temporal projection / merge / velocity
 *   - affine_zncc.wgsl:57-99 final ZNCC of a converged affine warp
 *   - spatial_seed.wgsl:40-52,65-190,268-309 translation hypothesis scoring
 *     (choose) and the affine frontier transport
 *
 * Rounding contract (shared with the CUDA kernels, which are written
 * independently to the same contract): every float operation is a single
 * IEEE-754 binary32 operation, rounded to nearest; a*b+c is only fused where
 * this file writes fmaf(); no expression is contracted by the compiler
 * (build with -ffp-contract=off).  The WGSL source leaves fusion and division
 * accuracy to the driver; this file fixes one admissible choice so that the
 * GPU kernels can be checked bit for bit.  Divisions by 6 in the cubic
 * weights are multiplications by the binary32 value of 1/6.
 *
 * Reductions: a subset's pixels are distributed over `lanes` lanes
 * (pixel = lane + k*lanes), each lane accumulates its own partial sums in
 * pixel order, and the lanes are combined by the pairwise tree of
 * icgn.wgsl:782-799 (stride lanes/2, lanes/4, ..., 1; lane i += lane i+stride).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MODEL_AFFINE 0
#define MODEL_TRANSLATION 1
#define MODEL_QUADRATIC 2
#define INTERP_BSPLINE 0
#define INTERP_LINEAR 1
#define INTERP_KEYS 2
#define MAX_LANES 128

typedef struct {
    int width, height;
    int grid_w, grid_h;
    int subset_size, subset_stride;
    int model, interp, lanes;
    int iterations;          /* 1..30 */
    float tolerance, zncc_min;
    int roi_enabled;         /* status -3 propagation for ROI-excluded windows */
    int divergence_patience; /* 0 disables the stagnation check */
    int divergence_min_iterations;
    const float *weights;    /* S*S integration weights, NULL = uniform */
    float weight_sum;        /* used when weights != NULL (metadata copy) */
} oracle_solve_cfg;

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* icgn.wgsl:128-143: one reflection without edge repetition, then clamp. */
static inline int mirror_clamp(int c, int n) {
    int r = c;
    if (c < 0) r = -c;
    else if (c >= n) r = 2 * n - 2 - c;
    return clampi(r, 0, n - 1);
}

/* icgn.wgsl:145-214.  fir25[k+12] is the tap at offset k (k=-12..12). */
void oracle_prefilter(const uint8_t *img, int W, int H, const float *fir25,
                      float *coef, float *scratch) {
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        const uint8_t *row = img + (size_t)y * W;
        for (int x = 0; x < W; ++x) {
            float acc = 0.0f;
            for (int k = -12; k <= 12; ++k)
                acc = fmaf(fir25[k + 12], (float)row[mirror_clamp(x + k, W)], acc);
            scratch[(size_t)y * W + x] = acc;
        }
    }
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            float acc = 0.0f;
            for (int k = -12; k <= 12; ++k)
                acc = fmaf(fir25[k + 12], scratch[(size_t)mirror_clamp(y + k, H) * W + x], acc);
            coef[(size_t)y * W + x] = acc;
        }
    }
}

static const float K6 = 1.0f / 6.0f;

/* icgn.wgsl:230-240 uniform cubic B-spline weights (Horner forms). */
static inline void bspline_weights(float t, float w[4]) {
    float t2 = t * t, t3 = t2 * t, s = 1.0f - t;
    w[0] = ((s * s) * s) * K6;
    w[1] = fmaf(fmaf(3.0f, t, -6.0f), t2, 4.0f) * K6;
    w[2] = fmaf(fmaf(fmaf(-3.0f, t, 3.0f), t, 3.0f), t, 1.0f) * K6;
    w[3] = t3 * K6;
}

/* icgn.wgsl:283-292 Keys cubic convolution weights, a = -0.5. */
static inline void keys_weights(float t, float w[4]) {
    float t2 = t * t;
    w[0] = fmaf(fmaf(-0.5f, t, 1.0f), t, -0.5f) * t;
    w[1] = fmaf(fmaf(1.5f, t, -2.5f), t2, 1.0f);
    w[2] = fmaf(fmaf(-1.5f, t, 2.0f), t, 0.5f) * t;
    w[3] = fmaf(0.5f, t, -0.5f) * t2;
}

/* 4x4 separable tensor gather; taps are clamped into the image so that a
 * bulging quadratic warp can never read outside the plane. */
static inline float gather16_f(const float *plane, int W, int H, int bx, int by,
                               const float wx[4], const float wy[4]) {
    int xs[4], ys[4];
    for (int i = 0; i < 4; ++i) {
        xs[i] = clampi(bx + i - 1, 0, W - 1);
        ys[i] = clampi(by + i - 1, 0, H - 1);
    }
    float value = 0.0f;
    for (int j = 0; j < 4; ++j) {
        const float *r = plane + (size_t)ys[j] * W;
        float row = 0.0f;
        for (int i = 0; i < 4; ++i) row = fmaf(wx[i], r[xs[i]], row);
        value = fmaf(wy[j], row, value);
    }
    return value;
}

static inline float gather16_u8(const uint8_t *img, int W, int H, int bx, int by,
                                const float wx[4], const float wy[4]) {
    int xs[4], ys[4];
    for (int i = 0; i < 4; ++i) {
        xs[i] = clampi(bx + i - 1, 0, W - 1);
        ys[i] = clampi(by + i - 1, 0, H - 1);
    }
    float value = 0.0f;
    for (int j = 0; j < 4; ++j) {
        const uint8_t *r = img + (size_t)ys[j] * W;
        float row = 0.0f;
        for (int i = 0; i < 4; ++i) row = fmaf(wx[i], (float)r[xs[i]], row);
        value = fmaf(wy[j], row, value);
    }
    return value;
}

/* WGSL mix(a, b, t) = a*(1-t) + b*t, fused on the last product. */
static inline float mixf(float a, float b, float t) { return fmaf(b, t, a * (1.0f - t)); }

/* icgn.wgsl:242-319 sample_target. */
static inline float sample_target(int interp, const float *coef, const uint8_t *img,
                                  int W, int H, float px, float py) {
    float fx = floorf(px), fy = floorf(py);
    int bx = (int)fx, by = (int)fy;
    float tx = px - fx, ty = py - fy;
    if (interp == INTERP_LINEAR) {
        int x0 = clampi(bx, 0, W - 1), x1 = clampi(bx + 1, 0, W - 1);
        int y0 = clampi(by, 0, H - 1), y1 = clampi(by + 1, 0, H - 1);
        float a = img[(size_t)y0 * W + x0], b = img[(size_t)y0 * W + x1];
        float c = img[(size_t)y1 * W + x0], d = img[(size_t)y1 * W + x1];
        return mixf(mixf(a, b, tx), mixf(c, d, tx), ty);
    }
    float wx[4], wy[4];
    if (interp == INTERP_KEYS) {
        keys_weights(tx, wx);
        keys_weights(ty, wy);
        return gather16_u8(img, W, H, bx, by, wx, wy);
    }
    bspline_weights(tx, wx);
    bspline_weights(ty, wy);
    return gather16_f(coef, W, H, bx, by, wx, wy);
}

typedef struct {
    float t[2];      /* tx, ty */
    float lin[4];    /* ux, uy, vx, vy */
    float curv[6];   /* uxx, uxy, uyy, vxx, vxy, vyy */
} warp_t;

/* Displacement at local (lx, ly); hx2 = lx*lx/2, xy = lx*ly, hy2 = ly*ly/2. */
static inline void displacement(int model, const warp_t *w, float lx, float ly,
                                float hx2, float xy, float hy2, float *dx, float *dy) {
    if (model == MODEL_TRANSLATION) {
        *dx = w->t[0];
        *dy = w->t[1];
        return;
    }
    float ax = w->t[0] + fmaf(w->lin[0], lx, w->lin[1] * ly);
    float ay = w->t[1] + fmaf(w->lin[2], lx, w->lin[3] * ly);
    if (model == MODEL_QUADRATIC) {
        ax = ax + fmaf(w->curv[0], hx2, fmaf(w->curv[1], xy, w->curv[2] * hy2));
        ay = ay + fmaf(w->curv[3], hx2, fmaf(w->curv[4], xy, w->curv[5] * hy2));
    }
    *dx = ax;
    *dy = ay;
}

/* icgn.wgsl:103-111 optional stagnation check; status 3 is internal. */
static inline float divergence_status(const oracle_solve_cfg *c, float change, unsigned count,
                                      float status, float *previous, unsigned *stalled) {
    if (c->divergence_patience == 0 || status != 0.0f) return status;
    if (count >= (unsigned)c->divergence_min_iterations)
        *stalled = (change >= *previous) ? *stalled + 1u : 0u;
    *previous = change;
    return (*stalled >= (unsigned)c->divergence_patience) ? 3.0f : status;
}

static inline float length2(float a, float b) { return sqrtf(fmaf(a, a, b * b)); }

/* icgn.wgsl:437-513 quadratic inverse composition through the lifted 6x6
 * warp matrix, pivoted Gauss-Jordan in binary32. Returns 0 when singular. */
static int compose_quadratic(warp_t *w, const float d[12]) {
    float u = d[0], ux = d[1], uy = d[2], v = d[3], vx = d[4], vy = d[5];
    float uxx = d[6], uxy = d[7], uyy = d[8], vxx = d[9], vxy = d[10], vyy = d[11];
    float m[6][12];
    memset(m, 0, sizeof m);
    /* Row 0..5 of the lifted warp matrix (icgn.wgsl:393-435), fused left to right. */
    m[0][0] = fmaf(u, uxx, fmaf(ux, ux, 1.0f + 2.0f * ux));
    m[0][1] = fmaf(2.0f * (1.0f + ux), uy, 2.0f * u * uxy);
    m[0][2] = fmaf(u, uyy, uy * uy);
    m[0][3] = 2.0f * u * (1.0f + ux);
    m[0][4] = 2.0f * u * uy;
    m[0][5] = u * u;
    m[1][0] = 0.5f * fmaf(u, vxx, fmaf(2.0f * (1.0f + ux), vx, v * uxx));
    m[1][1] = (fmaf(u, vxy, fmaf(v, uxy, fmaf(ux, vy, fmaf(uy, vx, 1.0f)))) + vy) + ux;
    m[1][2] = 0.5f * fmaf(u, vyy, fmaf(2.0f * uy, 1.0f + vy, v * uyy));
    m[1][3] = fmaf(u, vx, fmaf(v, ux, v));
    m[1][4] = fmaf(u, vy, fmaf(v, uy, u));
    m[1][5] = u * v;
    m[2][0] = fmaf(v, vxx, vx * vx);
    m[2][1] = fmaf(2.0f * vx, 1.0f + vy, 2.0f * v * vxy);
    m[2][2] = fmaf(v, vyy, fmaf(vy, vy, 1.0f + 2.0f * vy));
    m[2][3] = 2.0f * v * vx;
    m[2][4] = 2.0f * v * (1.0f + vy);
    m[2][5] = v * v;
    m[3][0] = 0.5f * uxx; m[3][1] = uxy; m[3][2] = 0.5f * uyy;
    m[3][3] = 1.0f + ux;  m[3][4] = uy;  m[3][5] = u;
    m[4][0] = 0.5f * vxx; m[4][1] = vxy; m[4][2] = 0.5f * vyy;
    m[4][3] = vx;         m[4][4] = 1.0f + vy; m[4][5] = v;
    m[5][0] = 0.0f; m[5][1] = 0.0f; m[5][2] = 0.0f; m[5][3] = 0.0f; m[5][4] = 0.0f; m[5][5] = 1.0f;
    for (int r = 0; r < 6; ++r) m[r][6 + r] = 1.0f;
    for (int col = 0; col < 6; ++col) {
        int prow = col;
        float psize = fabsf(m[col][col]);
        for (int cand = col + 1; cand < 6; ++cand) {
            float cs = fabsf(m[cand][col]);
            if (cs > psize) { prow = cand; psize = cs; }
        }
        if (psize < 1e-8f) return 0;
        if (prow != col) {
            float tmp[12];
            memcpy(tmp, m[col], sizeof tmp);
            memcpy(m[col], m[prow], sizeof tmp);
            memcpy(m[prow], tmp, sizeof tmp);
        }
        float pivot = m[col][col];
        for (int e = 0; e < 12; ++e) m[col][e] = m[col][e] / pivot;
        for (int r = 0; r < 6; ++r) {
            if (r == col) continue;
            float f = m[r][col];
            for (int e = 0; e < 12; ++e) m[r][e] = fmaf(-f, m[col][e], m[r][e]);
        }
    }
    float cu[6] = {0.5f * w->curv[0], w->curv[1], 0.5f * w->curv[2], 1.0f + w->lin[0], w->lin[1], w->t[0]};
    float cv[6] = {0.5f * w->curv[3], w->curv[4], 0.5f * w->curv[5], w->lin[2], 1.0f + w->lin[3], w->t[1]};
    float nu[6], nv[6];
    for (int col = 0; col < 6; ++col) {
        float au = 0.0f, av = 0.0f;
        for (int e = 0; e < 6; ++e) {
            au = fmaf(cu[e], m[e][6 + col], au);
            av = fmaf(cv[e], m[e][6 + col], av);
        }
        nu[col] = au;
        nv[col] = av;
    }
    w->curv[0] = 2.0f * nu[0]; w->curv[1] = nu[1]; w->curv[2] = 2.0f * nu[2];
    w->curv[3] = 2.0f * nv[0]; w->curv[4] = nv[1]; w->curv[5] = 2.0f * nv[2];
    w->t[0] = nu[5];
    w->t[1] = nv[5];
    w->lin[0] = nu[3] - 1.0f; w->lin[1] = nu[4];
    w->lin[2] = nv[3];        w->lin[3] = nv[4] - 1.0f;
    return 1;
}

static inline int parameter_count(int model) { return model == MODEL_QUADRATIC ? 12 : 6; }
static inline int state_stride(int model) { return model == MODEL_QUADRATIC ? 16 : 8; }
static inline int meta_stride(int model) { return model == MODEL_QUADRATIC ? 28 : 16; }

/* One subset: icgn.wgsl:595-958.  support / box (partial windows,
 * icgn.wgsl:1042-1085 with PARTIAL_SUPPORT): pixel bits of the window's
 * support and its (x0, y0, x1, y1) pixel box; NULL for complete windows. */
static void solve_one(const oracle_solve_cfg *c, int index, const uint8_t *img, const float *coef,
                      const float *refplane, const float *meta, const float *hinv,
                      const warp_t *initial, int enabled, int preserve_disabled, float *state,
                      const uint32_t *support, const float *box) {
    const int W = c->width, H = c->height, S = c->subset_size, st = c->subset_stride;
    const int model = c->model, L = c->lanes;
    const int n = parameter_count(model);
    const float *md = meta + (size_t)index * meta_stride(model);
    const float *hi = hinv + (size_t)index * n * n;
    warp_t w = *initial;
    if (model == MODEL_TRANSLATION) memset(w.lin, 0, sizeof w.lin);
    if (model != MODEL_QUADRATIC) memset(w.curv, 0, sizeof w.curv);
    int reference_valid = support ? md[1] == -4.0f : md[1] >= 0.5f;
    int valid = enabled && reference_valid;
    float rejected = -1.0f;
    if (c->roi_enabled && !support) rejected = fminf(-1.0f, md[1]);
    float status = valid ? 0.0f : rejected;
    float iters = 0.0f;
    const int gx = index % c->grid_w, gy = index / c->grid_w;
    const float half = 0.5f * ((float)S - 1.0f);
    const int mean_off = model == MODEL_QUADRATIC ? 26 : 14;
    const float ref_mean = (st != S || support) ? md[mean_off] : 0.0f;
    const float wsum = (c->weights || support) ? md[3 + 2 * n] : (float)(S * S);
    /* local extent checked against the image: the support box or the window */
    const float bx0 = support ? box[0] - half : -half, by0 = support ? box[1] - half : -half;
    const float bx1 = support ? box[2] - half : half, by1 = support ? box[3] - half : half;
    float previous_change = 3.402823e38f;
    unsigned stalled = 0;
    const int npix = S * S;

    for (int it = 0; it < 30; ++it) {
        if (!(c->divergence_patience != 0 && status == 3.0f)) {
            int inside = 1;
            if (model == MODEL_TRANSLATION) {
                float x0, y0, x1, y1;
                if (support) {
                    x0 = ((float)(gx * st) + box[0]) + w.t[0]; y0 = ((float)(gy * st) + box[1]) + w.t[1];
                    x1 = ((float)(gx * st) + box[2]) + w.t[0]; y1 = ((float)(gy * st) + box[3]) + w.t[1];
                } else {
                    x0 = (float)(gx * st) + w.t[0]; y0 = (float)(gy * st) + w.t[1];
                    x1 = (float)(gx * st + S - 1) + w.t[0]; y1 = (float)(gy * st + S - 1) + w.t[1];
                }
                inside = x0 >= 2.0f && y0 >= 2.0f && x1 <= (float)W - 3.0f && y1 <= (float)H - 3.0f;
            } else {
                int count = model == MODEL_QUADRATIC ? 9 : 4;
                for (int p = 0; p < count; ++p) {
                    float lx, ly;
                    if (model == MODEL_QUADRATIC) {
                        lx = (float)(p % 3 - 1) * half;
                        ly = (float)(p / 3 - 1) * half;
                    } else {
                        lx = (p == 1 || p == 3) ? bx1 : bx0;
                        ly = (p >= 2) ? by1 : by0;
                    }
                    float dx, dy;
                    displacement(model, &w, lx, ly, 0.5f * lx * lx, lx * ly, 0.5f * ly * ly, &dx, &dy);
                    float px = ((float)(gx * st) + (half + lx)) + dx;
                    float py = ((float)(gy * st) + (half + ly)) + dy;
                    inside = inside && px >= 2.0f && py >= 2.0f && px <= (float)W - 3.0f &&
                             py <= (float)H - 3.0f;
                }
            }
            if (!inside) {
                if (!c->roi_enabled || status > -2.5f) status = -1.0f;
            }
        }
        if (it >= c->iterations || fabsf(status) > 0.5f) break;

        float part[MAX_LANES][15];
        for (int lane = 0; lane < L; ++lane) {
            float s[15];
            for (int k = 0; k < 15; ++k) s[k] = 0.0f;
            for (int p = lane; p < npix; p += L) {
                if (support && !((support[p >> 5] >> (p & 31)) & 1u)) continue;
                int col = p % S, row = p / S;
                float lx = (float)col - half, ly = (float)row - half;
                float hx2 = 0.5f * lx * lx, xy = lx * ly, hy2 = 0.5f * ly * ly;
                float dx, dy;
                displacement(model, &w, lx, ly, hx2, xy, hy2, &dx, &dy);
                int pxi = gx * st + col, pyi = gy * st + row;
                float g = sample_target(c->interp, coef, img, W, H, (float)pxi + dx, (float)pyi + dy);
                const float *rv = refplane + ((size_t)pyi * W + pxi) * 4;
                float f = rv[0] - ref_mean;
                float wt = c->weights ? c->weights[p] : 1.0f;
                float wc = wt * g;
                float gxg = rv[1] * wc, gyg = rv[2] * wc;
                s[0] = s[0] + wc;
                s[1] = fmaf(wc, g, s[1]);
                s[2] = fmaf(wt * f, g, s[2]);
                s[3] = s[3] + gxg;
                s[6] = s[6] + gyg;
                if (model != MODEL_TRANSLATION) {
                    s[4] = fmaf(gxg, lx, s[4]);
                    s[5] = fmaf(gxg, ly, s[5]);
                    s[7] = fmaf(gyg, lx, s[7]);
                    s[8] = fmaf(gyg, ly, s[8]);
                    if (model == MODEL_QUADRATIC) {
                        s[9] = fmaf(gxg, hx2, s[9]);
                        s[10] = fmaf(gxg, xy, s[10]);
                        s[11] = fmaf(gxg, hy2, s[11]);
                        s[12] = fmaf(gyg, hx2, s[12]);
                        s[13] = fmaf(gyg, xy, s[13]);
                        s[14] = fmaf(gyg, hy2, s[14]);
                    }
                }
            }
            memcpy(part[lane], s, sizeof s);
        }
        for (int stride = L / 2; stride >= 1; stride /= 2)
            for (int lane = 0; lane < stride; ++lane)
                for (int k = 0; k < 15; ++k) part[lane][k] = part[lane][k] + part[lane + stride][k];
        const float *t = part[0];
        /* t: 0 sum g, 1 sum g^2, 2 sum f g, 3..8 J^T g (gx, gx x, gx y, gy, gy x, gy y), 9..14 quadratic */
        float jg[12] = {t[3], t[4], t[5], t[6], t[7], t[8], t[9], t[10], t[11], t[12], t[13], t[14]};
        float mean_g = t[0] / wsum;
        float norm_g = sqrtf(fmaxf(0.0f, fmaf(-t[0], mean_g, t[1])));
        float norm_f = md[0];
        iters = (float)(it + 1);
        if (norm_g < 1e-9f || norm_f < 1e-9f) {
            status = -2.0f;
            continue;
        }
        float ratio = norm_f / norm_g;
        const int sum_off = 2 + n;
        float res[12], delta[12];
        for (int k = 0; k < 12; ++k) { res[k] = 0.0f; delta[k] = 0.0f; }
        if (model == MODEL_TRANSLATION) {
            res[0] = fmaf(-ratio, fmaf(-mean_g, md[sum_off + 0], jg[0]), md[2 + 0]);
            res[3] = fmaf(-ratio, fmaf(-mean_g, md[sum_off + 3], jg[3]), md[2 + 3]);
            float a0 = hi[0 * 6 + 0] * res[0];
            a0 = fmaf(hi[0 * 6 + 3], res[3], a0);
            float a3 = hi[3 * 6 + 0] * res[0];
            a3 = fmaf(hi[3 * 6 + 3], res[3], a3);
            delta[0] = -a0;
            delta[3] = -a3;
        } else {
            for (int k = 0; k < n; ++k)
                res[k] = fmaf(-ratio, fmaf(-mean_g, md[sum_off + k], jg[k]), md[2 + k]);
            for (int r = 0; r < n; ++r) {
                float a = 0.0f;
                for (int k = 0; k < n; ++k) a = fmaf(hi[r * n + k], res[k], a);
                delta[r] = -a;
            }
        }
        float change;
        if (model == MODEL_QUADRATIC) {
            if (!compose_quadratic(&w, delta)) {
                status = -1.0f;
                continue;
            }
            change = 0.0f;
            for (int p = 0; p < 9; ++p) {
                float x = (float)(p % 3 - 1) * half, y = (float)(p / 3 - 1) * half;
                float hx2 = 0.5f * x * x, xy = x * y, hy2 = 0.5f * y * y;
                float a = fmaf(delta[2], y, fmaf(delta[1], x, delta[0]));
                a = a + fmaf(delta[6], hx2, fmaf(delta[7], xy, delta[8] * hy2));
                float b = fmaf(delta[5], y, fmaf(delta[4], x, delta[3]));
                b = b + fmaf(delta[9], hx2, fmaf(delta[10], xy, delta[11] * hy2));
                change = fmaxf(change, length2(a, b));
            }
        } else {
            float det = 1.0f;
            if (model == MODEL_AFFINE) det = fmaf(1.0f + delta[1], 1.0f + delta[5], -(delta[2] * delta[4]));
            if (fabsf(det) < 1e-8f) {
                status = -1.0f;
                continue;
            }
            if (model == MODEL_TRANSLATION) {
                w.t[0] = w.t[0] - delta[0];
                w.t[1] = w.t[1] - delta[3];
                change = length2(delta[0], delta[3]);
            } else {
                float i11 = (1.0f + delta[5]) / det, i12 = -delta[2] / det;
                float i21 = -delta[4] / det, i22 = (1.0f + delta[1]) / det;
                float w11 = 1.0f + w.lin[0], w12 = w.lin[1], w21 = w.lin[2], w22 = 1.0f + w.lin[3];
                float itx = -fmaf(i11, delta[0], i12 * delta[3]);
                float ity = -fmaf(i21, delta[0], i22 * delta[3]);
                w.t[0] = w.t[0] + fmaf(w11, itx, w12 * ity);
                w.t[1] = w.t[1] + fmaf(w21, itx, w22 * ity);
                float u11 = fmaf(w11, i11, w12 * i21), u12 = fmaf(w11, i12, w12 * i22);
                float u21 = fmaf(w21, i11, w22 * i21), u22 = fmaf(w21, i12, w22 * i22);
                w.lin[0] = u11 - 1.0f; w.lin[1] = u12; w.lin[2] = u21; w.lin[3] = u22 - 1.0f;
                change = 0.0f;
                for (int p = 0; p < 4; ++p) {
                    float x = (p == 1 || p == 3) ? half : -half;
                    float y = (p >= 2) ? half : -half;
                    float a = fmaf(delta[2], y, fmaf(delta[1], x, delta[0]));
                    float b = fmaf(delta[5], y, fmaf(delta[4], x, delta[3]));
                    change = fmaxf(change, length2(a, b));
                }
            }
        }
        float zncc = t[2] / (norm_f * norm_g);
        float conv = (change >= c->tolerance) ? 0.0f : (zncc >= c->zncc_min ? 1.0f : -2.0f);
        status = divergence_status(c, change, (unsigned)(it + 1), conv, &previous_change, &stalled);
    }
    if (enabled || !preserve_disabled) {
        float final_status = (c->divergence_patience != 0 && status == 3.0f) ? 0.0f : status;
        float *o = state + (size_t)index * state_stride(model);
        o[0] = w.t[0]; o[1] = w.lin[0]; o[2] = w.lin[1]; o[3] = w.t[1];
        if (model == MODEL_QUADRATIC) {
            o[4] = w.lin[2]; o[5] = w.lin[3]; o[6] = w.curv[0]; o[7] = w.curv[1];
            o[8] = w.curv[2]; o[9] = w.curv[3]; o[10] = w.curv[4]; o[11] = w.curv[5];
            o[12] = final_status; o[13] = iters; o[14] = 0.0f; o[15] = 0.0f;
        } else {
            o[4] = w.lin[2]; o[5] = w.lin[3]; o[6] = final_status; o[7] = iters;
        }
    }
}

/* Entry for solve (seed == NULL: zero seed, all enabled), solve_seeded and
 * retry_seeded (icgn.wgsl:960-1017).  `subsets` restricts work to a list of
 * indices (NULL = the whole grid). */
void oracle_solve(const oracle_solve_cfg *c, const uint8_t *img, const float *coef,
                  const float *refplane, const float *meta, const float *hinv,
                  const float *seed_state, const uint32_t *active, int preserve_disabled,
                  const int32_t *subsets, int subset_count, float *state) {
    const int count = subsets ? subset_count : c->grid_w * c->grid_h;
    const int ss = state_stride(c->model);
    #pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < count; ++k) {
        int index = subsets ? subsets[k] : k;
        warp_t w;
        memset(&w, 0, sizeof w);
        int enabled = 1;
        if (seed_state) {
            const float *s = seed_state + (size_t)index * ss;
            w.t[0] = s[0]; w.lin[0] = s[1]; w.lin[1] = s[2]; w.t[1] = s[3];
            w.lin[2] = s[4]; w.lin[3] = s[5];
            if (c->model == MODEL_QUADRATIC)
                for (int j = 0; j < 6; ++j) w.curv[j] = s[6 + j];
            enabled = active[index] != 0u;
        }
        solve_one(c, index, img, coef, refplane, meta, hinv, &w, enabled, preserve_disabled, state, NULL, NULL);
    }
}

/* Partial windows (solve_partial / solve_partial_seeded, icgn.wgsl:1062-1078):
 * window indices[k] with support words words[k * words_per] and box
 * boxes[4 k]; seed_state / active as for oracle_solve (NULL: zero seed). */
void oracle_solve_partial(const oracle_solve_cfg *c, const uint8_t *img, const float *coef, const float *refplane,
                          const float *meta, const float *hinv, const float *seed_state, const uint32_t *active,
                          const int32_t *indices, int count, const uint32_t *words, int words_per, const float *boxes,
                          float *state) {
    const int ss = state_stride(c->model);
    #pragma omp parallel for schedule(dynamic, 4)
    for (int k = 0; k < count; ++k) {
        int index = indices[k];
        warp_t w;
        memset(&w, 0, sizeof w);
        int enabled = 1;
        if (seed_state) {
            const float *s = seed_state + (size_t)index * ss;
            w.t[0] = s[0]; w.lin[0] = s[1]; w.lin[1] = s[2]; w.t[1] = s[3];
            w.lin[2] = s[4]; w.lin[3] = s[5];
            enabled = active[index] != 0u;
        }
        solve_one(c, index, img, coef, refplane, meta, hinv, &w, enabled, 0, state, words + (size_t)k * words_per,
                  boxes + 4 * (size_t)k);
    }
}

/* ------------------------------------------------------------------ UOD */

/* icgn.wgsl:1087-1101: bubble passes, then the middle value(s). */
static float median_nine(float *v, int count) {
    for (int phase = 0; phase < 9; ++phase)
        for (int i = 0; i < 8; ++i)
            if (i + 1 < count && v[i] > v[i + 1]) {
                float s = v[i];
                v[i] = v[i + 1];
                v[i + 1] = s;
            }
    if (count % 2 == 1) return v[count / 2];
    return 0.5f * (v[count / 2 - 1] + v[count / 2]);
}

/* icgn.wgsl:1103-1148 Hoare quickselect (order statistic; exact). */
static float select_rank(float *v, int count, int rank) {
    int low = 0, high = count - 1;
    for (;;) {
        if (low >= high) return v[rank];
        float pivot = v[low + (high - low) / 2];
        int left = low, right = high;
        for (;;) {
            while (left <= high && v[left] < pivot) ++left;
            while (right >= low && v[right] > pivot) --right;
            if (left > right) break;
            float s = v[left]; v[left] = v[right]; v[right] = s;
            ++left; --right;
        }
        if (rank <= right) high = right;
        else if (rank >= left) low = left;
        else return v[rank];
    }
}

static float median_81(float *v, int count) {
    if (count % 2 == 1) return select_rank(v, count, count / 2);
    float lo = select_rank(v, count, count / 2 - 1);
    float hi = select_rank(v, count, count / 2);
    return 0.5f * (lo + hi);
}

/* icgn.wgsl:1150-1190 Taylor recentring of a neighbour's component. */
static float recentered(int model, const float *s, int comp, float ox, float oy) {
    if (model == MODEL_QUADRATIC) {
        switch (comp) {
        case 0: return fmaf(s[8], 0.5f * oy * oy, fmaf(s[7], ox * oy, fmaf(s[6], 0.5f * ox * ox, fmaf(s[2], oy, fmaf(s[1], ox, s[0])))));
        case 1: return fmaf(s[7], oy, fmaf(s[6], ox, s[1]));
        case 2: return fmaf(s[8], oy, fmaf(s[7], ox, s[2]));
        case 3: return fmaf(s[11], 0.5f * oy * oy, fmaf(s[10], ox * oy, fmaf(s[9], 0.5f * ox * ox, fmaf(s[5], oy, fmaf(s[4], ox, s[3])))));
        case 4: return fmaf(s[10], oy, fmaf(s[9], ox, s[4]));
        case 5: return fmaf(s[11], oy, fmaf(s[10], ox, s[5]));
        default: return s[comp];
        }
    }
    switch (comp) {
    case 0: return fmaf(s[2], oy, fmaf(s[1], ox, s[0]));
    case 3: return fmaf(s[5], oy, fmaf(s[4], ox, s[3]));
    default: return s[comp];
    }
}

typedef struct {
    int grid_w, grid_h;
    int subset_stride;
    int model;
    int policy;          /* 0 flag, 1 replace, 3 median */
    int median_size;     /* 3, 5, 7, 9 (median policy) */
    int scope_all;       /* median policy: smooth accepted subsets too */
    int seed_mode;       /* median_filter_seed entry: rejected fills become status 0 */
    int roi_enabled;
    const float *permissions; /* 4 floats per subset (ROI tail) or NULL */
    const float *meta;        /* metadata rows (validity in column 1) */
} oracle_uod_cfg;

static const int COMPONENT_ORDER[12] = {0, 3, 1, 2, 4, 5, 6, 7, 8, 9, 10, 11};

static int neighbour_allowed(const oracle_uod_cfg *c, int index, int dx, int dy, int wide) {
    if (!c->roi_enabled) return 1;
    const float *perm = c->permissions + (size_t)index * 4;
    unsigned bit, word;
    if (wide) {
        bit = (unsigned)((dy + 4) * 9 + dx + 4);
        word = (unsigned)perm[bit / 24];
    } else {
        bit = (unsigned)((dy + 1) * 3 + dx + 1);
        word = (unsigned)perm[0];
    }
    return (word & (1u << (bit % 24))) != 0;
}

/* icgn.wgsl:1192-1323 median repair (and optional smoothing). */
static void median_motion(const oracle_uod_cfg *c, int index, const float *state, float *out) {
    const int ss = state_stride(c->model);
    const float *own = state + (size_t)index * ss;
    float *dst = out + (size_t)index * ss;
    memcpy(dst, own, sizeof(float) * ss);
    int status_at = c->model == MODEL_QUADRATIC ? 12 : 6;
    float own_status = own[status_at];
    float ref_status = c->meta[(size_t)index * meta_stride(c->model) + 1];
    if ((own_status >= 0.5f && !c->scope_all) || (ref_status < 0.5f && ref_status != -4.0f)) return;
    int px = index % c->grid_w, py = index / c->grid_w;
    int radius = c->median_size / 2;
    int active = c->model == MODEL_TRANSLATION ? 2 : (c->model == MODEL_QUADRATIC ? 12 : 6);
    float filtered[12];
    for (int k = 0; k < 12; ++k) filtered[k] = own[k];
    for (int ai = 0; ai < active; ++ai) {
        int comp = COMPONENT_ORDER[ai];
        float values[81];
        int count = 0;
        if (own_status >= 0.5f) values[count++] = recentered(c->model, own, comp, 0.0f, 0.0f);
        for (int dy = -radius; dy <= radius; ++dy)
            for (int dx = -radius; dx <= radius; ++dx) {
                if (dx == 0 && dy == 0) continue;
                int nx = px + dx, ny = py + dy;
                if (nx < 0 || ny < 0 || nx >= c->grid_w || ny >= c->grid_h) continue;
                if (!neighbour_allowed(c, index, dx, dy, c->median_size > 3)) continue;
                const float *ns = state + ((size_t)ny * c->grid_w + nx) * ss;
                if (ns[status_at] < 0.5f) continue;
                values[count++] = recentered(c->model, ns, comp, -(float)c->subset_stride * (float)dx,
                                             -(float)c->subset_stride * (float)dy);
            }
        int minimum = (c->roi_enabled && c->median_size == 3 && own_status < 0.5f) ? 3 : 4;
        if (count < minimum) return;
        filtered[comp] = median_81(values, count);
    }
    for (int k = 0; k < 12 && k < ss; ++k) dst[k] = filtered[k];
    if (c->model == MODEL_QUADRATIC) {
        dst[12] = (c->seed_mode && own_status < 0.5f) ? 0.0f : own[12];
        dst[13] = own[13]; dst[14] = own[14]; dst[15] = own[15];
    } else {
        dst[6] = (c->seed_mode && own_status < 0.5f) ? 0.0f : own[6];
        dst[7] = own[7];
    }
}

/* icgn.wgsl:1325-1593 UOD flag / replace. */
static void uod_one(const oracle_uod_cfg *c, int index, const float *state, float *out) {
    if (c->policy == 3) {
        median_motion(c, index, state, out);
        return;
    }
    const int ss = state_stride(c->model);
    const float *own = state + (size_t)index * ss;
    float *dst = out + (size_t)index * ss;
    memcpy(dst, own, sizeof(float) * ss);
    int status_at = c->model == MODEL_QUADRATIC ? 12 : 6;
    if (own[status_at] < 0.5f) return;
    int px = index % c->grid_w, py = index / c->grid_w;
    int ncomp = c->model == MODEL_QUADRATIC ? 12 : 6;
    float nb[9][12];
    int count = 0;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            if (dx == 0 && dy == 0) continue;
            int nx = px + dx, ny = py + dy;
            if (nx < 0 || ny < 0 || nx >= c->grid_w || ny >= c->grid_h) continue;
            if (c->model != MODEL_QUADRATIC && !neighbour_allowed(c, index, dx, dy, 0)) continue;
            const float *ns = state + ((size_t)ny * c->grid_w + nx) * ss;
            if (ns[status_at] < 0.5f) continue;
            float ox = -(float)c->subset_stride * (float)dx, oy = -(float)c->subset_stride * (float)dy;
            for (int k = 0; k < ncomp; ++k) nb[count][k] = recentered(c->model, ns, k, ox, oy);
            ++count;
        }
    if (count < 4) return;
    float filtered[12], medians[12], values[9];
    for (int k = 0; k < 12; ++k) filtered[k] = medians[k] = (k < ncomp) ? own[k] : 0.0f;
    int model_components = c->model == MODEL_TRANSLATION ? 2 : ncomp;
    int median_count = c->policy == 1 ? model_components : 2;
    for (int ai = 0; ai < median_count; ++ai) {
        int comp = COMPONENT_ORDER[ai];
        for (int i = 0; i < count; ++i) values[i] = nb[i][comp];
        medians[comp] = median_nine(values, count);
    }
    int flagged = 0;
    for (int ai = 0; ai < 2; ++ai) {
        int comp = COMPONENT_ORDER[ai];
        for (int i = 0; i < count; ++i) values[i] = fabsf(nb[i][comp] - medians[comp]);
        float spread = median_nine(values, count);
        float score = fabsf(filtered[comp] - medians[comp]) / (spread + 0.1f);
        if (score > 2.0f) flagged = 1;
    }
    if (!flagged) return;
    if (c->policy == 1)
        for (int ai = 0; ai < model_components; ++ai) filtered[COMPONENT_ORDER[ai]] = medians[COMPONENT_ORDER[ai]];
    for (int k = 0; k < ncomp; ++k) dst[k] = filtered[k];
    if (c->model == MODEL_QUADRATIC) {
        dst[12] = 2.0f; dst[13] = own[13]; dst[14] = 0.0f; dst[15] = 0.0f;
    } else {
        dst[6] = 2.0f; dst[7] = own[7];
    }
}

void oracle_uod(const oracle_uod_cfg *c, const float *state, float *out) {
    const int count = c->grid_w * c->grid_h;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < count; ++i) uod_one(c, i, state, out);
}

/* ------------------------------------------------------------ pyramid */

/* full_pyramid.wgsl:218-249: integer 5x5 [1 4 6 4 1]^2 sum, reflected
 * source, truncating division by 256. */
void oracle_reduce(const uint8_t *src, int W, int H, uint8_t *dst) {
    const int w2 = W / 2, h2 = H / 2;
    static const unsigned taps[5] = {1u, 4u, 6u, 4u, 1u};
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < h2; ++y)
        for (int x = 0; x < w2; ++x) {
            unsigned acc = 0u;
            for (int j = 0; j < 5; ++j) {
                int sy = mirror_clamp(2 * y + j - 2, H);
                for (int i = 0; i < 5; ++i) {
                    int sx = mirror_clamp(2 * x + i - 2, W);
                    acc += taps[j] * taps[i] * (unsigned)src[(size_t)sy * W + sx];
                }
            }
            dst[(size_t)y * w2 + x] = (uint8_t)(acc / 256u);
        }
}

typedef struct {
    int src_grid_w, src_grid_h;
    int dst_grid_w, dst_grid_h;
    float src_scale, dst_scale;
    float subset_size, subset_stride;
    int model;
    int track_availability;
} oracle_seed_cfg;

/* full_pyramid.wgsl:251-308 */
static void accumulate_seed(const oracle_seed_cfg *c, const float *src, int sidx, float weight,
                            float spx, float spy, float dpx, float dpy, float tscale,
                            float a[4], float b[4], float cc[4], float *wsum) {
    const int ss = state_stride(c->model);
    const float *s = src + (size_t)sidx * ss;
    float status = c->model == MODEL_QUADRATIC ? s[12] : s[6];
    if (status < -0.5f) return;
    float dx = dpx - spx, dy = dpy - spy;
    float tu = fmaf(s[2], dy, fmaf(s[1], dx, s[0]));
    float tv = fmaf(s[5], dy, fmaf(s[4], dx, s[3]));
    float ux = s[1], uy = s[2], vx = s[4], vy = s[5];
    if (c->model == MODEL_QUADRATIC) {
        tu = tu + fmaf(s[8], 0.5f * dy * dy, fmaf(s[7], dx * dy, s[6] * (0.5f * dx * dx)));
        tv = tv + fmaf(s[11], 0.5f * dy * dy, fmaf(s[10], dx * dy, s[9] * (0.5f * dx * dx)));
        ux = ux + fmaf(s[7], dy, s[6] * dx);
        uy = uy + fmaf(s[8], dy, s[7] * dx);
        vx = vx + fmaf(s[10], dy, s[9] * dx);
        vy = vy + fmaf(s[11], dy, s[10] * dx);
    }
    a[0] = fmaf(weight * tu, tscale, a[0]);
    a[1] = fmaf(weight, ux, a[1]);
    a[2] = fmaf(weight, uy, a[2]);
    a[3] = fmaf(weight * tv, tscale, a[3]);
    b[0] = fmaf(weight, vx, b[0]);
    b[1] = fmaf(weight, vy, b[1]);
    if (c->model == MODEL_QUADRATIC) {
        float cs = 1.0f / tscale;
        b[2] = fmaf(weight * s[6], cs, b[2]);
        b[3] = fmaf(weight * s[7], cs, b[3]);
        for (int k = 0; k < 4; ++k) cc[k] = fmaf(weight * s[8 + k], cs, cc[k]);
    }
    *wsum = *wsum + weight;
}

/* full_pyramid.wgsl:310-395; returns the weight sum and writes a,b,c. */
static float interpolate_seed(const oracle_seed_cfg *c, const float *src, int didx,
                              unsigned perm, float a[4], float b[4], float cc[4]) {
    for (int k = 0; k < 4; ++k) a[k] = b[k] = cc[k] = 0.0f;
    float wsum = 0.0f;
    int dxg = didx % c->dst_grid_w, dyg = didx / c->dst_grid_w;
    float soff = (1.0f - c->src_scale) * 0.5f, doff = (1.0f - c->dst_scale) * 0.5f;
    float dcx = fmaf(c->subset_stride, (float)dxg, 0.5f * c->subset_size);
    float dcy = fmaf(c->subset_stride, (float)dyg, 0.5f * c->subset_size);
    float scx = fmaf(c->dst_scale, dcx, doff - soff) / c->src_scale;
    float scy = fmaf(c->dst_scale, dcy, doff - soff) / c->src_scale;
    float gxf = (scx - 0.5f * c->subset_size) / c->subset_stride;
    float gyf = (scy - 0.5f * c->subset_size) / c->subset_stride;
    int maxx = c->src_grid_w - 2 > 0 ? c->src_grid_w - 2 : 0;
    int maxy = c->src_grid_h - 2 > 0 ? c->src_grid_h - 2 : 0;
    int lx = clampi((int)floorf(gxf), 0, maxx), ly = clampi((int)floorf(gyf), 0, maxy);
    float fx = fminf(fmaxf(gxf - (float)lx, 0.0f), 1.0f);
    float fy = fminf(fmaxf(gyf - (float)ly, 0.0f), 1.0f);
    float tscale = c->src_scale / c->dst_scale;
    for (int corner = 0; corner < 4; ++corner) {
        if ((perm & (1u << corner)) == 0u) continue;
        int ox = corner & 1, oy = corner >> 1;
        int sx = lx + ox, sy = ly + oy;
        if (sx >= c->src_grid_w || sy >= c->src_grid_h) continue;
        float wx = ox ? fx : 1.0f - fx, wy = oy ? fy : 1.0f - fy;
        float spx = fmaf(c->subset_stride, (float)sx, 0.5f * c->subset_size);
        float spy = fmaf(c->subset_stride, (float)sy, 0.5f * c->subset_size);
        accumulate_seed(c, src, sy * c->src_grid_w + sx, wx * wy, spx, spy, scx, scy, tscale, a, b, cc, &wsum);
    }
    unsigned fallback = perm >> 5;
    if (wsum == 0.0f && fallback != 0u) {
        int sidx = (int)fallback - 1;
        const float *s = src + (size_t)sidx * state_stride(c->model);
        float st = c->model == MODEL_QUADRATIC ? s[12] : s[6];
        if (st >= 0.5f) {
            int sx = sidx % c->src_grid_w, sy = sidx / c->src_grid_w;
            float spx = fmaf(c->subset_stride, (float)sx, 0.5f * c->subset_size);
            float spy = fmaf(c->subset_stride, (float)sy, 0.5f * c->subset_size);
            accumulate_seed(c, src, sidx, 1.0f, spx, spy, scx, scy, tscale, a, b, cc, &wsum);
        }
    }
    if (wsum > 0.0f)
        for (int k = 0; k < 4; ++k) { a[k] = a[k] / wsum; b[k] = b[k] / wsum; cc[k] = cc[k] / wsum; }
    return wsum;
}

/* full_pyramid.wgsl:397-433.  perms == NULL: every destination uses 31.
 * weights (or NULL) receives each destination's weight sum. */
void oracle_transfer_seed(const oracle_seed_cfg *c, const float *src, const uint32_t *perms,
                          float *dst_seed, uint32_t *dst_active, float *weights) {
    const int count = c->dst_grid_w * c->dst_grid_h;
    const int ss = state_stride(c->model);
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < count; ++i) {
        unsigned perm = perms ? perms[i] : 31u;
        float a[4], b[4], cc[4];
        float wsum = interpolate_seed(c, src, i, perm, a, b, cc);
        float *d = dst_seed + (size_t)i * ss;
        for (int k = 0; k < 4; ++k) { d[k] = a[k]; d[4 + k] = b[k]; }
        if (c->model == MODEL_QUADRATIC) {
            for (int k = 0; k < 4; ++k) { d[8 + k] = cc[k]; d[12 + k] = 0.0f; }
        }
        if (c->track_availability) {
            float marker = wsum >= 0.99999f ? 0.0f : -1.0f;
            d[c->model == MODEL_QUADRATIC ? 12 : 6] = marker;
        }
        dst_active[i] = (perm >> 4) & 1u;
        if (weights) weights[i] = wsum;
    }
}

/* full_pyramid.wgsl:452-506 (refine_temporal_seed).  src = coarse accepted
 * history, src_ages its ages; history / ages = the fine accepted history;
 * dst_seed holds the ordinary transfer (with availability markers). */
void oracle_refine_temporal_seed(const oracle_seed_cfg *c, const float *src, const uint32_t *src_ages,
                                 const uint32_t *perms, const float *history, const uint32_t *ages,
                                 unsigned max_age, float *dst_seed, const uint32_t *dst_active) {
    const int count = c->dst_grid_w * c->dst_grid_h;
    const int ss = state_stride(c->model);
    const int status_at = c->model == MODEL_QUADRATIC ? 12 : 6;
    for (int i = 0; i < count; ++i) {
        if (dst_active[i] == 0u) continue;
        unsigned age = ages[i];
        if (age == 0xffffffffu || age > max_age) continue;
        float *d = dst_seed + (size_t)i * ss;
        if (d[status_at] < -0.5f) continue;
        unsigned perm = perms ? perms[i] : 31u;
        /* lower corner of the bilinear stencil, as in interpolate_seed */
        int dxg = i % c->dst_grid_w, dyg = i / c->dst_grid_w;
        float soff = (1.0f - c->src_scale) * 0.5f, doff = (1.0f - c->dst_scale) * 0.5f;
        float scx = fmaf(c->dst_scale, fmaf(c->subset_stride, (float)dxg, 0.5f * c->subset_size), doff - soff) / c->src_scale;
        float scy = fmaf(c->dst_scale, fmaf(c->subset_stride, (float)dyg, 0.5f * c->subset_size), doff - soff) / c->src_scale;
        int maxx = c->src_grid_w - 2 > 0 ? c->src_grid_w - 2 : 0;
        int maxy = c->src_grid_h - 2 > 0 ? c->src_grid_h - 2 : 0;
        int lx = clampi((int)floorf((scx - 0.5f * c->subset_size) / c->subset_stride), 0, maxx);
        int ly = clampi((int)floorf((scy - 0.5f * c->subset_size) / c->subset_stride), 0, maxy);
        int same = 1;
        for (int corner = 0; corner < 4 && same; ++corner) {
            if ((perm & (1u << corner)) == 0u) continue;
            int sx = lx + (corner & 1), sy = ly + (corner >> 1);
            if (sx >= c->src_grid_w || sy >= c->src_grid_h) continue;
            if (src_ages[sy * c->src_grid_w + sx] != age) same = 0;
        }
        if (!same) continue;
        float a[4], b[4], cc[4];
        float wsum = interpolate_seed(c, src, i, perm, a, b, cc);
        if (wsum < 0.99999f) continue;
        const float *h = history + (size_t)i * ss;
        float predicted[12] = {a[0], a[1], a[2], a[3], b[0], b[1], b[2], b[3], cc[0], cc[1], cc[2], cc[3]};
        int n = c->model == MODEL_QUADRATIC ? 12 : 6;
        for (int k = 0; k < n; ++k) d[k] = h[k] + (d[k] - predicted[k]);
    }
}

/* ------------------------------------------------------------ temporal */

/* full_pyramid.wgsl:508-554; returns 1 when the history accepted an update. */
void oracle_temporal_merge(int count, int model, unsigned max_age, int use_filtered,
                           float *history, uint32_t *ages, const float *raw, const float *output,
                           uint32_t *accepted_updates, uint32_t *expired) {
    const int ss = state_stride(model);
    const int status_at = model == MODEL_QUADRATIC ? 12 : 6;
    uint32_t acc = 0, exp_count = 0;
    for (int i = 0; i < count; ++i) {
        float rs = raw[(size_t)i * ss + status_at], fs = output[(size_t)i * ss + status_at];
        int raw_ok = rs == 1.0f || rs == 2.0f, fin_ok = fs == 1.0f || fs == 2.0f;
        if (fin_ok && (use_filtered || raw_ok)) {
            const float *src = use_filtered ? output : raw;
            memcpy(history + (size_t)i * ss, src + (size_t)i * ss, sizeof(float) * ss);
            ages[i] = 0u;
            ++acc;
        } else if (ages[i] != 0xffffffffu) {
            uint32_t age = (ages[i] < 0xfffffffdu ? ages[i] : 0xfffffffdu) + 1u;
            ages[i] = age;
            if (age > max_age) {
                history[(size_t)i * ss + status_at] = -1.0f;
                if (age == max_age + 1u) ++exp_count;
            }
        }
    }
    if (accepted_updates) *accepted_updates = acc;
    if (expired) *expired = exp_count;
}

/* full_pyramid.wgsl:83-109 velocity prediction; returns the predicted count. */
uint32_t oracle_temporal_predict(int count, int model, const float *current, const float *previous,
                                 const uint32_t *cur_ages, const uint32_t *prev_ages, float *out) {
    const int ss = state_stride(model);
    const int status_at = model == MODEL_QUADRATIC ? 12 : 6;
    const int status_vec = model == MODEL_QUADRATIC ? 12 : 4;
    uint32_t predicted = 0;
    for (int i = 0; i < count; ++i) {
        const float *c = current + (size_t)i * ss, *p = previous + (size_t)i * ss;
        float *o = out + (size_t)i * ss;
        int predict = cur_ages[i] == 0u && prev_ages[i] == 0u && c[status_at] >= 0.5f && p[status_at] >= 0.5f;
        for (int k = 0; k < ss; ++k) o[k] = predict ? fmaf(2.0f, c[k], -p[k]) : c[k];
        /* The status vector is copied as a measurement; its first two
         * entries are the dv/dx, dv/dy parameters for the 8-float layout. */
        for (int k = 0; k < 4; ++k) o[status_vec + k] = c[status_vec + k];
        if (model != MODEL_QUADRATIC && predict) {
            o[4] = fmaf(2.0f, c[4], -p[4]);
            o[5] = fmaf(2.0f, c[5], -p[5]);
        }
        predicted += (uint32_t)predict;
    }
    return predicted;
}

/* full_pyramid.wgsl:126-148 */
void oracle_temporal_save_previous(int count, int model, const float *history, const uint32_t *ages,
                                   const float *raw, const float *output, float *prev_history,
                                   uint32_t *prev_ages) {
    const int ss = state_stride(model);
    const int status_at = model == MODEL_QUADRATIC ? 12 : 6;
    for (int i = 0; i < count; ++i) {
        float rs = raw[(size_t)i * ss + status_at], fs = output[(size_t)i * ss + status_at];
        if ((rs == 1.0f || rs == 2.0f) && (fs == 1.0f || fs == 2.0f)) {
            memcpy(prev_history + (size_t)i * ss, history + (size_t)i * ss, sizeof(float) * ss);
            prev_ages[i] = ages[i];
        } else if (prev_ages[i] != 0xffffffffu) {
            prev_ages[i] = (prev_ages[i] < 0xfffffffdu ? prev_ages[i] : 0xfffffffdu) + 1u;
        }
    }
}

/* ------------------------------------------------------- ZNCC seed search */

/* Exhaustive integer-shift ZNCC search (the CUDA seed search restated):
 * for every subset (or, with only_missing, every subset whose seed status
 * slot is -1), the shift (dx, dy) in [-R, R]^2 maximising
 *   (n Sfg - Sf Sg) / sqrt((n Sff - Sf^2)(n Sgg - Sg^2))
 * over exact integer sums of the 8-bit windows, lowest row-major index on
 * ties; windows leaving the image are skipped.  Writes a translation seed
 * and activity 1 (ROI-excluded subsets: zero seed, activity 0). */
/* centered: shifts around the rounded seed translation; mask (or NULL):
 * search only subsets whose byte is non-zero. */
void oracle_seed_search_ex(const uint8_t *ref, const uint8_t *tgt, int W, int H, int grid_w, int grid_h, int S,
                           int stride, int R, int model, int only_missing, const uint8_t *selected, float *seed,
                           uint32_t *active, float *score, int centered, const uint8_t *mask) {
    const int ss = state_stride(model), sat = model == MODEL_QUADRATIC ? 12 : 6;
    const int count = grid_w * grid_h, side = 2 * R + 1;
    #pragma omp parallel for schedule(dynamic, 4)
    for (int idx = 0; idx < count; ++idx) {
        float *sd = seed + (size_t)idx * ss;
        if (only_missing && sd[sat] != -1.0f) continue;
        if (mask && !mask[idx]) continue;
        int cx0 = 0, cy0 = 0;
        if (centered) {
            cx0 = fabsf(sd[0]) <= (float)W ? (int)rintf(sd[0]) : 0;
            cy0 = fabsf(sd[3]) <= (float)H ? (int)rintf(sd[3]) : 0;
        }
        const int rx0 = (idx % grid_w) * stride, ry0 = (idx / grid_w) * stride;
        const int px0 = rx0 + cx0, py0 = ry0 + cy0;
        if (selected && !selected[idx]) {
            if (!only_missing) {
                for (int k = 0; k < ss; ++k) sd[k] = 0.0f;
                active[idx] = 0u;
                if (score) score[idx] = -2.0f;
            }
            continue;
        }
        long long sf = 0, sff = 0;
        for (int r = 0; r < S; ++r)
            for (int c = 0; c < S; ++c) {
                const long long f = ref[(size_t)(ry0 + r) * W + rx0 + c];
                sf += f;
                sff += f * f;
            }
        const long long n = (long long)S * S, vf = n * sff - sf * sf;
        double best = -3.0;
        int best_cand = -1;
        for (int cand = 0; cand < side * side; ++cand) {
            const int dy = cand / side - R, dx = cand % side - R;
            if (px0 + dx < 0 || py0 + dy < 0 || px0 + dx + S - 1 > W - 1 || py0 + dy + S - 1 > H - 1) continue;
            long long sg = 0, sgg = 0, sfg = 0;
            for (int r = 0; r < S; ++r)
                for (int c = 0; c < S; ++c) {
                    const long long g = tgt[(size_t)(py0 + dy + r) * W + px0 + dx + c];
                    const long long f = ref[(size_t)(ry0 + r) * W + rx0 + c];
                    sg += g;
                    sgg += g * g;
                    sfg += f * g;
                }
            const long long vg = n * sgg - sg * sg;
            double s = -2.0;
            if (vf > 0 && vg > 0) s = (double)(n * sfg - sf * sg) / sqrt((double)vf * (double)vg);
            if (s > best) {
                best = s;
                best_cand = cand;
            }
        }
        for (int k = 0; k < ss; ++k) sd[k] = 0.0f;
        if (best_cand >= 0 && best > -1.5) {
            sd[0] = (float)(cx0 + best_cand % side - R);
            sd[3] = (float)(cy0 + best_cand / side - R);
        }
        active[idx] = 1u;
        if (score) score[idx] = (float)best;
    }
}

void oracle_seed_search(const uint8_t *ref, const uint8_t *tgt, int W, int H, int grid_w, int grid_h, int S,
                        int stride, int R, int model, int only_missing, const uint8_t *selected, float *seed,
                        uint32_t *active, float *score) {
    oracle_seed_search_ex(ref, tgt, W, H, grid_w, grid_h, S, stride, R, model, only_missing, selected, seed, active,
                          score, 0, NULL);
}

/* ------------------------------------------------------------ final ZNCC */

/* affine_zncc.wgsl:57-99 with `lanes` lanes; -2 marks unavailable. */
void oracle_final_zncc(int W, int H, int grid_w, int grid_h, int S, int st, int interp, int lanes,
                       const uint8_t *img, const float *coef, const float *refplane,
                       const float *state, float *out) {
    const int count = grid_w * grid_h;
    #pragma omp parallel for schedule(static)
    for (int index = 0; index < count; ++index) {
        const float *p = state + (size_t)index * 8;
        if (p[6] != 1.0f) { out[index] = -2.0f; continue; }
        int gx = index % grid_w, gy = index / grid_w;
        float half = ((float)S - 1.0f) * 0.5f;
        float part[MAX_LANES][6];
        for (int lane = 0; lane < lanes; ++lane) {
            float s[6] = {0, 0, 0, 0, 0, 0};
            for (int k = lane; k < S * S; k += lanes) {
                int col = k % S, row = k / S;
                int px = gx * st + col, py = gy * st + row;
                float lx = (float)col - half, ly = (float)row - half;
                float tx = (float)px + (p[0] + fmaf(p[1], lx, p[2] * ly));
                float ty = (float)py + (p[3] + fmaf(p[4], lx, p[5] * ly));
                if (tx >= 2.0f && ty >= 2.0f && tx <= (float)(W - 3) && ty <= (float)(H - 3)) {
                    float g = sample_target(interp, coef, img, W, H, tx, ty);
                    float f = refplane[((size_t)py * W + px) * 4];
                    s[0] = s[0] + f;
                    s[1] = s[1] + g;
                    s[2] = fmaf(f, f, s[2]);
                    s[3] = fmaf(g, g, s[3]);
                    s[4] = fmaf(f, g, s[4]);
                    s[5] = s[5] + 1.0f;
                }
            }
            memcpy(part[lane], s, sizeof s);
        }
        for (int stride = lanes / 2; stride >= 1; stride /= 2)
            for (int lane = 0; lane < stride; ++lane)
                for (int k = 0; k < 6; ++k) part[lane][k] = part[lane][k] + part[lane + stride][k];
        float *s = part[0];
        float n = s[5];
        float nn = fmaxf(n, 1.0f);
        float vf = s[2] - s[0] * s[0] / nn;
        float vg = s[3] - s[1] * s[1] / nn;
        if (n == (float)(S * S) && vf > 1e-9f && vg > 1e-9f) {
            float r = (s[4] - s[0] * s[1] / n) / sqrtf(vf * vg);
            out[index] = fminf(fmaxf(r, -1.0f), 1.0f);
        } else {
            out[index] = -2.0f;
        }
    }
}

/* ------------------------------------------------------------ spatial seeds */

/* spatial_seed.wgsl:40-52: insertion sort, mean of the two middle values. */
static float spatial_median(float *v, int n) {
    for (int i = 1; i < n; ++i) {
        float value = v[i];
        int j = i;
        while (j > 0 && !(v[j - 1] <= value)) {
            v[j] = v[j - 1];
            --j;
        }
        v[j] = value;
    }
    return 0.5f * (v[(n - 1) / 2] + v[n / 2]);
}

/* spatial_seed.wgsl:268-309 affine_frontier.  states / seeds: 8 floats per
 * subset; active receives 1 for every new frontier subset. */
void oracle_affine_frontier(int count, int grid_w, int stride, const float *snap, const uint32_t *perms,
                            float *seeds, uint32_t *active) {
    const int gh = count / grid_w;
    for (int index = 0; index < count; ++index) {
        if ((perms[index] & 16u) == 0u) continue;
        if (snap[8 * index + 6] >= 0.5f) continue;
        int gx = index % grid_w, gy = index / grid_w;
        float t0[9], g0[9], g1[9], t1[9], g2[9], g3[9];
        int n = 0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                if (dx == 0 && dy == 0) continue;
                int x = gx + dx, y = gy + dy, bit = (dy + 1) * 3 + dx + 1;
                if (x < 0 || y < 0 || x >= grid_w || y >= gh || (perms[index] & (1u << bit)) == 0u) continue;
                int nb = y * grid_w + x;
                const float *p = snap + 8 * nb;
                if ((perms[nb] & 16u) == 0u || p[6] != 1.0f) continue;
                float ddx = (float)(-dx) * (float)stride, ddy = (float)(-dy) * (float)stride;
                t0[n] = p[0] + (p[1] * ddx + p[2] * ddy);
                t1[n] = p[3] + (p[4] * ddx + p[5] * ddy);
                g0[n] = p[1]; g1[n] = p[2]; g2[n] = p[4]; g3[n] = p[5];
                ++n;
            }
        if (n == 0) continue;
        float *d = seeds + 8 * index;
        d[0] = spatial_median(t0, n); d[1] = spatial_median(g0, n);
        d[2] = spatial_median(g1, n); d[3] = spatial_median(t1, n);
        d[4] = spatial_median(g2, n); d[5] = spatial_median(g3, n);
        d[6] = 0.0f; d[7] = 0.0f;
        active[index] = 1u;
    }
}

static float unorm8(uint8_t b) { return (float)b / 255.0f; }

static float spatial_linear(const uint8_t *img, int W, float x, float y) {
    float fx = floorf(x), fy = floorf(y);
    int ix = (int)fx, iy = (int)fy;
    float tx = x - fx, ty = y - fy;
    const uint8_t *r0 = img + (size_t)iy * W + ix, *r1 = r0 + W;
    float a = unorm8(r0[0]), b = unorm8(r0[1]), c = unorm8(r1[0]), e = unorm8(r1[1]);
    float top = a * (1.0f - tx) + b * tx;
    float bottom = c * (1.0f - tx) + e * tx;
    return 255.0f * (top * (1.0f - ty) + bottom * ty) - 128.0f;
}

/* spatial_seed.wgsl:65-190 choose (no score cache): 64 lane-strided partial
 * sums per hypothesis and the halving pairwise tree. */
void oracle_spatial_choose(const uint8_t *ref, const uint8_t *tgt, int W, int H, int grid_w, int count, int S,
                           int stride, int sample_step, float min_gain, float min_displacement, int failed_only,
                           int candidate_mode, const float *snap, const float *prior, const uint32_t *perms,
                           float *seeds, float *scores, uint32_t *active) {
    const int gh = count / grid_w;
    #pragma omp parallel for schedule(dynamic, 16)
    for (int index = 0; index < count; ++index) {
        uint32_t perm = perms[index];
        if ((perm & 16u) == 0u) continue;
        if (failed_only && snap[8 * index + 6] >= 0.5f) continue;
        int gx = index % grid_w, gy = index / grid_w;
        float ownx = snap[8 * index + 0], owny = snap[8 * index + 3];
        float cand[11][3];
        for (int k = 0; k < 11; ++k) cand[k][0] = cand[k][1] = cand[k][2] = 0.0f;
        cand[0][0] = ownx; cand[0][1] = owny; cand[0][2] = 1.0f;
        cand[1][0] = prior ? prior[8 * index + 0] : 0.0f;
        cand[1][1] = prior ? prior[8 * index + 3] : 0.0f;
        cand[1][2] = 1.0f;
        float us[9], vs[9];
        int n = 0, slot = 2;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                int bit = (dy + 1) * 3 + dx + 1, x = gx + dx, y = gy + dy;
                int inside = x >= 0 && y >= 0 && x < grid_w && y < gh;
                if (inside && (perm & (1u << bit)) != 0u) {
                    int nb = y * grid_w + x;
                    if ((perms[nb] & 16u) != 0u) {
                        float px = snap[8 * nb + 0], py = snap[8 * nb + 3];
                        if ((dx != 0 || dy != 0) && candidate_mode != 1) {
                            cand[slot][0] = px; cand[slot][1] = py; cand[slot][2] = 1.0f;
                        }
                        if (snap[8 * nb + 6] >= 0.5f) { us[n] = px; vs[n] = py; ++n; }
                    }
                }
                if (dx != 0 || dy != 0) ++slot;
            }
        if (candidate_mode != 0 && n > 0) {
            cand[10][0] = spatial_median(us, n); cand[10][1] = spatial_median(vs, n); cand[10][2] = 1.0f;
        }
        float bx = ownx, by = owny, brho = -2.0f, bown = -2.0f;
        float ox = (float)(gx * stride), oy = (float)(gy * stride);
        int side = (S + sample_step - 1) / sample_step, total = side * side;
        float ftotal = (float)total;
        for (int k = 0; k < 11; ++k) {
            float cx = cand[k][0], cy = cand[k][1];
            float minx = ox + cx, miny = oy + cy;
            float maxx = minx + (float)(S - 1), maxy = miny + (float)(S - 1);
            if (cand[k][2] == 0.0f || !(fabsf(cx) <= 1e12f && fabsf(cy) <= 1e12f) || minx < 2.0f || miny < 2.0f ||
                maxx > (float)(W - 3) || maxy > (float)(H - 3))
                continue;
            float sx[64], sy[64], sz[64], sw[64], sg[64];
            for (int lane = 0; lane < 64; ++lane) {
                float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f, g2 = 0.0f;
                for (int pixel = lane; pixel < total; pixel += 64) {
                    float offx = (float)(pixel % side) * (float)sample_step;
                    float offy = (float)(pixel / side) * (float)sample_step;
                    int rx = (int)(ox + offx), ry = (int)(oy + offy);
                    float f = 255.0f * unorm8(ref[(size_t)ry * W + rx]) - 128.0f;
                    float g = spatial_linear(tgt, W, (ox + offx) + cx, (oy + offy) + cy);
                    a0 = a0 + f; a1 = a1 + g; a2 = a2 + f * g; a3 = a3 + f * f; g2 = g2 + g * g;
                }
                sx[lane] = a0; sy[lane] = a1; sz[lane] = a2; sw[lane] = a3; sg[lane] = g2;
            }
            for (int off = 32; off > 0; off >>= 1)
                for (int lane = 0; lane < off; ++lane) {
                    sx[lane] = sx[lane] + sx[lane + off]; sy[lane] = sy[lane] + sy[lane + off];
                    sz[lane] = sz[lane] + sz[lane + off]; sw[lane] = sw[lane] + sw[lane + off];
                    sg[lane] = sg[lane] + sg[lane + off];
                }
            float vf = fmaxf(0.0f, sw[0] - sx[0] * sx[0] / ftotal);
            float vg = fmaxf(0.0f, sg[0] - sy[0] * sy[0] / ftotal);
            float rho = -2.0f;
            if (vf > 1e-9f && vg > 1e-9f) rho = (sz[0] - sx[0] * sy[0] / ftotal) / sqrtf(vf * vg);
            if (k == 0) bown = rho;
            if (rho > brho) { bx = cx; by = cy; brho = rho; }
        }
        float ddx = bx - ownx, ddy = by - owny;
        int improved = brho > bown + min_gain && sqrtf(ddx * ddx + ddy * ddy) > min_displacement;
        scores[4 * index + 0] = bown; scores[4 * index + 1] = brho;
        scores[4 * index + 2] = improved ? 1.0f : 0.0f; scores[4 * index + 3] = 0.0f;
        if (improved) {
            float *d = seeds + 8 * index;
            d[0] = bx; d[1] = 0.0f; d[2] = 0.0f; d[3] = by;
            d[4] = d[5] = d[6] = d[7] = 0.0f;
            active[index] = 1u;
        }
    }
}
