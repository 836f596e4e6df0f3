/* FP64 restatement of the differentiable shading model and its adjoint (TEST INFRASTRUCTURE ONLY).
 *
 * The reference renders with quantised barycentrics (source/main.c:1092-1102), which are piecewise
 * constant in the vertex positions, so their gradient is zero almost everywhere. The
 * differentiable path therefore shades, under the visibility the exact rasteriser produced (one
 * input triangle per pixel, fixed), with continuous barycentrics at the reference's sample point
 * (the pixel corner, main.c:1014), and interpolates like the reference does for w = 1 (linear
 * barycentrics, main.c:1118-1160). The shader is vertex colour times the bilinear texel of an
 * RGBA32F texture, with the reference's bilinear_f addressing and weights
 * (common_shader_core.h:143-161); positions are passthrough screen coordinates in [0,1]
 * (passthrough_vs.c:20-23): X = W * x, Y = H * (1 - y).
 *
 * This file is the oracle the GPU adjoint is checked against, and it is itself checked against
 * central finite differences (tests/test_adjoint_oracle.py).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "oracle.h"

/* The differentiable coverage (malevich_gb300/csrc/adjoint.cu): a covered pixel counts when its
 * corner's continuous barycentrics are all >= -1/8; a frozen cell of CELL_DROPPED marks a pixel
 * the rule (evaluated in single precision) dropped. */
#define MIN_BARYCENTRIC (-0.125)
#define CELL_DROPPED INT32_MIN

typedef struct {
    double l[3];           /* barycentrics */
    double col[3], tex[3]; /* interpolated colour, filtered texel */
    double fs, ft;         /* bilinear fractions */
    int32_t s0, t0;        /* bilinear cell */
    double A;              /* twice the signed screen-space area */
    double X[3], Y[3];     /* screen-space vertices */
    uint32_t vi[3];
} pix_state;

static inline double tex_at(const orc_diff_scene *s, int32_t i, int32_t j, int c) {
    i = i < 0 ? 0 : (i > (int32_t)s->tw - 1 ? (int32_t)s->tw - 1 : i);
    j = j < 0 ? 0 : (j > (int32_t)s->th - 1 ? (int32_t)s->th - 1 : j);
    return s->tex[((size_t)j * s->tw + (size_t)i) * 4 + c];
}

/* Evaluates one covered pixel; returns 0 if the differentiable coverage drops it. */
static int eval_pixel(const orc_diff_scene *s, const orc_diff_view *v, uint32_t px, uint32_t py, uint32_t t,
                      const int32_t *cell, pix_state *ps) {
    const double W = (double)v->width, H = (double)v->height;
    for (int k = 0; k < 3; ++k) {
        uint32_t vi = s->ib[3 * (size_t)t + k];
        ps->vi[k] = vi;
        ps->X[k] = W * v->pos[2 * (size_t)vi];
        ps->Y[k] = H * (1.0 - v->pos[2 * (size_t)vi + 1]);
    }
    const double x = (double)px, y = (double)py;
    if (cell && cell[0] == CELL_DROPPED) return 0;
    ps->A = (ps->X[1] - ps->X[0]) * (ps->Y[2] - ps->Y[0]) - (ps->X[2] - ps->X[0]) * (ps->Y[1] - ps->Y[0]);
    if (ps->A == 0.0) return 0;
    /* lambda_k = cross(v_{k+1} - p, v_{k+2} - p) / A */
    for (int k = 0; k < 3; ++k) {
        int a = (k + 1) % 3, b = (k + 2) % 3;
        ps->l[k] = ((ps->X[a] - x) * (ps->Y[b] - y) - (ps->Y[a] - y) * (ps->X[b] - x)) / ps->A;
    }
    if (!cell && (ps->l[0] < MIN_BARYCENTRIC || ps->l[1] < MIN_BARYCENTRIC || ps->l[2] < MIN_BARYCENTRIC)) return 0;
    double u = 0, vv = 0;
    for (int c = 0; c < 3; ++c) ps->col[c] = 0;
    for (int k = 0; k < 3; ++k) {
        for (int c = 0; c < 3; ++c) ps->col[c] += ps->l[k] * s->col[3 * (size_t)ps->vi[k] + c];
        u += ps->l[k] * s->uv[2 * (size_t)ps->vi[k]];
        vv += ps->l[k] * s->uv[2 * (size_t)ps->vi[k] + 1];
    }
    const double sf = (double)s->tw * u - 0.5, tf = (double)s->th * (1.0 - vv) - 0.5;
    ps->s0 = cell ? cell[0] : (int32_t)floor(sf);
    ps->t0 = cell ? cell[1] : (int32_t)floor(tf);
    ps->fs = sf - (double)ps->s0;
    ps->ft = tf - (double)ps->t0;
    for (int c = 0; c < 3; ++c) {
        double a = (1 - ps->fs) * tex_at(s, ps->s0, ps->t0, c) + ps->fs * tex_at(s, ps->s0 + 1, ps->t0, c);
        double b = (1 - ps->fs) * tex_at(s, ps->s0, ps->t0 + 1, c) + ps->fs * tex_at(s, ps->s0 + 1, ps->t0 + 1, c);
        ps->tex[c] = (1 - ps->ft) * a + ps->ft * b;
    }
    return 1;
}

double orc_diff_loss(const orc_diff_scene *s, const orc_diff_view *views, uint32_t nviews, double *image) {
    double loss = 0.0;
    for (uint32_t vi = 0; vi < nviews; ++vi) {
        const orc_diff_view *v = views + vi;
        for (uint32_t py = 0; py < v->height; ++py)
            for (uint32_t px = 0; px < v->width; ++px) {
                const size_t p = (size_t)py * v->width + px;
                const uint32_t t = v->prim[p];
                if (t == 0xFFFFFFFFu) continue;
                pix_state ps;
                const int in = eval_pixel(s, v, px, py, t, v->cells ? v->cells + 2 * p : NULL, &ps);
                for (int c = 0; c < 3; ++c) {
                    double o = in ? ps.col[c] * ps.tex[c] : 0.0; /* a dropped pixel shades to 0 */
                    if (image) image[((size_t)vi * v->width * v->height + p) * 3 + c] = o;
                    double d = o - v->target[p * 3 + c];
                    loss += d * d;
                }
            }
    }
    return loss;
}

void orc_diff_cells(const orc_diff_scene *s, const orc_diff_view *v, int32_t *cells) {
    for (uint32_t py = 0; py < v->height; ++py)
        for (uint32_t px = 0; px < v->width; ++px) {
            const size_t p = (size_t)py * v->width + px;
            pix_state ps;
            cells[2 * p] = cells[2 * p + 1] = 0;
            if (v->prim[p] == 0xFFFFFFFFu) continue;
            if (!eval_pixel(s, v, px, py, v->prim[p], NULL, &ps)) {
                cells[2 * p] = cells[2 * p + 1] = CELL_DROPPED;
                continue;
            }
            cells[2 * p] = ps.s0;
            cells[2 * p + 1] = ps.t0;
        }
}

/* a d - b c by Kahan's FMA algorithm, as the GPU kernels compute it (Jeannerod, Louvet and Muller,
 * Math. Comp. 2013). */
static inline float det2f(float a, float b, float c, float d) {
    const float w = b * c;
    const float e = fmaf(-b, c, w);
    const float f = fmaf(a, d, -w);
    return f + e;
}

/* The bilinear cell each pixel falls in, and the differentiable coverage, computed with the GPU
 * kernels' single-precision operation sequence (malevich_gb300/csrc/adjoint.cu: corner_geometry,
 * the barycentric division and shade's exact split of the texel coordinate). The cell is a discrete choice: the loss is
 * continuous across cell boundaries but its derivative in the positions jumps there, so the FP64
 * adjoint is compared with the GPU under the GPU's own cells. Compiled with -ffp-contract=off so
 * every operation rounds like the kernel's (built with --fmad=false; fmaf where it calls fmaf). */
void orc_diff_cells_f32(const orc_diff_scene *s, const orc_diff_view *v, int32_t *cells) {
    const float W = (float)v->width, H = (float)v->height;
    const float tw = (float)s->tw, th = (float)s->th;
    for (uint32_t py = 0; py < v->height; ++py)
        for (uint32_t px = 0; px < v->width; ++px) {
            const size_t p = (size_t)py * v->width + px;
            const uint32_t t = v->prim[p];
            cells[2 * p] = cells[2 * p + 1] = 0;
            if (t == 0xFFFFFFFFu) continue;
            uint32_t vi[3];
            float ppx[3], ppy[3];
            for (int k = 0; k < 3; ++k) {
                vi[k] = s->ib[3 * (size_t)t + k];
                ppx[k] = (float)v->pos[2 * (size_t)vi[k]];
                ppy[k] = (float)v->pos[2 * (size_t)vi[k] + 1];
            }
            const float x = (float)px, y = (float)py, hy = H - y;
            const float ax = fmaf(W, ppx[0], -x), ay = fmaf(-H, ppy[0], hy);
            const float bx = fmaf(W, ppx[1], -x), by = fmaf(-H, ppy[1], hy);
            const float cx = fmaf(W, ppx[2], -x), cy = fmaf(-H, ppy[2], hy);
            const float e1x = W * (ppx[1] - ppx[0]), e1y = H * (ppy[0] - ppy[1]);
            const float e2x = W * (ppx[2] - ppx[0]), e2y = H * (ppy[0] - ppy[2]);
            const float A = det2f(e1x, e2x, e1y, e2y);
            cells[2 * p] = cells[2 * p + 1] = CELL_DROPPED;
            if (A == 0.0f) continue;
            const float l1 = det2f(cx, cy, ax, ay) / A;
            const float l2 = det2f(ax, ay, bx, by) / A;
            const float l0 = 1.0f - l1 - l2;
            if (l0 < -0.125f || l1 < -0.125f || l2 < -0.125f) continue;
            float u[3], w[3];
            for (int k = 0; k < 3; ++k) {
                u[k] = (float)s->uv[2 * (size_t)vi[k]];
                w[k] = (float)s->uv[2 * (size_t)vi[k] + 1];
            }
            const float ps = tw * u[0], pse = fmaf(tw, u[0], -ps);
            const float bs = ps - 0.5f, fbs = floorf(bs);
            const float q = th * w[0], qe = fmaf(th, w[0], -q);
            const float a = th - 0.5f, r = a - q, rb = r - a;
            const float re = (a - (r - rb)) + (-q - rb);
            const float fbt = floorf(r);
            const float rs = ((bs - fbs) + pse) + (l1 * (tw * (u[1] - u[0])) + l2 * (tw * (u[2] - u[0])));
            const float rt = ((r - fbt) + (re - qe)) - (l1 * (th * (w[1] - w[0])) + l2 * (th * (w[2] - w[0])));
            cells[2 * p] = (int32_t)fbs + (int32_t)floorf(rs);
            cells[2 * p + 1] = (int32_t)fbt + (int32_t)floorf(rt);
        }
}

/* Adds dL/dcol, dL/dtex and dL/dpos (per view) of the L2 loss to the given arrays. */
void orc_diff_grad(const orc_diff_scene *s, const orc_diff_view *views, uint32_t nviews, double *g_col,
                   double *g_tex, double *g_pos) {
    for (uint32_t vi = 0; vi < nviews; ++vi) {
        const orc_diff_view *v = views + vi;
        const double W = (double)v->width, H = (double)v->height;
        double *gp = g_pos ? g_pos + (size_t)vi * s->n_verts * 2 : NULL;
        for (uint32_t py = 0; py < v->height; ++py)
            for (uint32_t px = 0; px < v->width; ++px) {
                const size_t p = (size_t)py * v->width + px;
                const uint32_t t = v->prim[p];
                if (t == 0xFFFFFFFFu) continue;
                pix_state ps;
                if (!eval_pixel(s, v, px, py, t, v->cells ? v->cells + 2 * p : NULL, &ps)) continue;
                double dout[3], dcol[3], dtex[3];
                for (int c = 0; c < 3; ++c) {
                    dout[c] = 2.0 * (ps.col[c] * ps.tex[c] - v->target[p * 3 + c]);
                    dcol[c] = dout[c] * ps.tex[c];
                    dtex[c] = dout[c] * ps.col[c];
                }
                /* vertex colours */
                if (g_col)
                    for (int k = 0; k < 3; ++k)
                        for (int c = 0; c < 3; ++c) g_col[3 * (size_t)ps.vi[k] + c] += ps.l[k] * dcol[c];
                /* texels, through the bilinear weights */
                const double w00 = (1 - ps.fs) * (1 - ps.ft), w10 = ps.fs * (1 - ps.ft);
                const double w01 = (1 - ps.fs) * ps.ft, w11 = ps.fs * ps.ft;
                const int32_t si[4] = {ps.s0, ps.s0 + 1, ps.s0, ps.s0 + 1}, ti[4] = {ps.t0, ps.t0, ps.t0 + 1, ps.t0 + 1};
                const double wt[4] = {w00, w10, w01, w11};
                if (g_tex)
                    for (int q = 0; q < 4; ++q) {
                        int32_t i = si[q] < 0 ? 0 : (si[q] > (int32_t)s->tw - 1 ? (int32_t)s->tw - 1 : si[q]);
                        int32_t j = ti[q] < 0 ? 0 : (ti[q] > (int32_t)s->th - 1 ? (int32_t)s->th - 1 : ti[q]);
                        for (int c = 0; c < 3; ++c) g_tex[((size_t)j * s->tw + i) * 4 + c] += wt[q] * dtex[c];
                    }
                if (!gp) continue;
                /* positions: through the bilinear fractions and the barycentrics */
                double dfs = 0, dft = 0;
                for (int c = 0; c < 3; ++c) {
                    double t00 = tex_at(s, ps.s0, ps.t0, c), t10 = tex_at(s, ps.s0 + 1, ps.t0, c);
                    double t01 = tex_at(s, ps.s0, ps.t0 + 1, c), t11 = tex_at(s, ps.s0 + 1, ps.t0 + 1, c);
                    dfs += dtex[c] * ((1 - ps.ft) * (t10 - t00) + ps.ft * (t11 - t01));
                    dft += dtex[c] * (((1 - ps.fs) * t01 + ps.fs * t11) - ((1 - ps.fs) * t00 + ps.fs * t10));
                }
                const double du = dfs * (double)s->tw, dv = -dft * (double)s->th;
                double G[3];
                for (int k = 0; k < 3; ++k) {
                    const uint32_t q = ps.vi[k];
                    G[k] = du * s->uv[2 * (size_t)q] + dv * s->uv[2 * (size_t)q + 1];
                    for (int c = 0; c < 3; ++c) G[k] += dcol[c] * s->col[3 * (size_t)q + c];
                }
                const double x = (double)px, y = (double)py;
                double S = G[0] * ps.l[0] + G[1] * ps.l[1] + G[2] * ps.l[2];
                double gX[3], gY[3];
                const double *X = ps.X, *Y = ps.Y, A = ps.A;
                /* d lambda_k / d v_j (numerators cross(v_{k+1}-p, v_{k+2}-p)), minus S dA/dv_j */
                gX[0] = (G[1] * (-(Y[2] - y)) + G[2] * (Y[1] - y)) / A - S * (-(Y[2] - Y[0]) + (Y[1] - Y[0])) / A;
                gY[0] = (G[1] * (X[2] - x) + G[2] * (-(X[1] - x))) / A - S * ((X[2] - X[0]) - (X[1] - X[0])) / A;
                gX[1] = (G[0] * (Y[2] - y) + G[2] * (-(Y[0] - y))) / A - S * (Y[2] - Y[0]) / A;
                gY[1] = (G[0] * (-(X[2] - x)) + G[2] * (X[0] - x)) / A - S * (-(X[2] - X[0])) / A;
                gX[2] = (G[0] * (-(Y[1] - y)) + G[1] * (Y[0] - y)) / A - S * (-(Y[1] - Y[0])) / A;
                gY[2] = (G[0] * (X[1] - x) + G[1] * (-(X[0] - x))) / A - S * (X[1] - X[0]) / A;
                for (int k = 0; k < 3; ++k) {
                    gp[2 * (size_t)ps.vi[k]] += W * gX[k];
                    gp[2 * (size_t)ps.vi[k] + 1] += -H * gY[k];
                }
            }
    }
}
