/*
 * CPU oracle of the neural-LoD hot path -- TEST INFRASTRUCTURE ONLY (see nlod_oracle.h).
 * Build: oracle/build.py (gcc -O2 -ffp-contract=off -fopenmp -shared).
 */
#include "nlod_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------------------------------
 * Grid layout: grid.h:195-204 (scale/resolution) and 982-1015 (offset table).
 * ------------------------------------------------------------------------------------------- */
uint32_t orc_grid_offsets(int n_levels, uint32_t log2_hashmap_size, uint32_t base_resolution, float per_level_scale,
                          int kind, uint32_t* offsets, uint32_t* res, float* scale) {
    const float log2s = log2f(per_level_scale);
    uint32_t off = 0;
    for (int i = 0; i < n_levels; ++i) {
        const float s = exp2f((float)i * log2s) * (float)base_resolution - 1.0f;
        const uint32_t r = (uint32_t)ceilf(s) + 1u;
        const uint32_t max_params = 0xFFFFFFFFu / 2u;
        uint32_t p;
        if (powf((float)r, 3.0f) > (float)max_params) p = max_params;
        else p = r * r * r;
        p = (p + 7u) / 8u * 8u;
        if (kind == 2) {
            uint32_t t = base_resolution * base_resolution * base_resolution;
            if (t < p) p = t;
        } else if (kind == 0) {
            uint32_t t = 1u << log2_hashmap_size;
            if (t < p) p = t;
        }
        offsets[i] = off;
        if (res) res[i] = r;
        if (scale) scale[i] = s;
        off += p;
    }
    offsets[n_levels] = off;
    return off;
}

/* grid.h:111-187 */
static uint32_t orc_hash(int kind, uint32_t x, uint32_t y, uint32_t z) {
    if (kind == 0) return (x * 1u) ^ (y * 2654435761u) ^ (z * 805459861u);
    if (kind == 1) return (x * 1958374283u) ^ (y * 2654435761u) ^ (z * 805459861u);
    return (x * 2165219737u) ^ (y * 1434869437u) ^ (z * 2097192037u);
}

static uint32_t orc_grid_index(const OrcGrid* g, int level, const uint32_t pos[3]) {
    const uint32_t size = g->offset[level + 1] - g->offset[level];
    uint32_t stride = 1, index = 0;
    for (int dim = 0; dim < 3 && stride <= size; ++dim) {
        index += pos[dim] * stride;
        stride *= g->res[level];
    }
    if (g->kind == 0 && size < stride) index = orc_hash(g->hash, pos[0], pos[1], pos[2]);
    return index % size;
}

/* common_device.h:437-464 with FP32 arithmetic: p = x*scale + 0.5 (fused), cell = floor(p). */
static void orc_pos_fract(float x, float scale, float* frac, uint32_t* cell) {
    const float p = fmaf(x, scale, 0.5f);
    const float fl = floorf(p);
    *cell = (uint32_t)(int)fl;
    *frac = p - fl;
}

static double orc_interp(int interp, double t) { return interp == 2 ? t * t * (3.0 - 2.0 * t) : t; }

static int orc_masked_fwd(int level, float ml_frac, int n_levels) {
    const float max_level = (ml_frac * (float)(n_levels * 2)) / 2.0f;
    return (float)level >= max_level + 1e-3f;
}
static int orc_skipped_bwd(int level, float ml_frac, int n_levels) {
    const float max_level = (ml_frac * (float)(n_levels * 2)) / 2.0f;
    return (float)level > max_level + 1e-3f;
}

/* Corner entries (table indices within the level) and weights of one level. Returns corners. */
static int orc_corners(const OrcGrid* g, int level, const float p[3], uint32_t entries[8], double weights[8]) {
    float frac[3];
    uint32_t cell[3];
    for (int d = 0; d < 3; ++d) orc_pos_fract(p[d], g->scale[level], &frac[d], &cell[d]);
    if (g->interp == 1) {
        entries[0] = orc_grid_index(g, level, cell);
        weights[0] = 1.0;
        return 1;
    }
    double t[3];
    for (int d = 0; d < 3; ++d) t[d] = orc_interp(g->interp, (double)frac[d]);
    for (int c = 0; c < 8; ++c) {
        uint32_t q[3];
        double w = 1.0;
        for (int d = 0; d < 3; ++d) {
            if (c & (1 << d)) { w *= t[d]; q[d] = cell[d] + 1u; }
            else { w *= 1.0 - t[d]; q[d] = cell[d]; }
        }
        entries[c] = orc_grid_index(g, level, q);
        weights[c] = w;
    }
    return 8;
}

/* ---------------------------------------------------------------------------------------------
 * Spherical harmonics by recurrence: Y_l^m = K_l^m Pbar_l^m(z) * {sqrt2 Re, sqrt2 Im, 1}((x+iy)^|m|)
 * with Pbar_l^m = P_l^m / sin^m (Condon-Shortley phase included).
 * ------------------------------------------------------------------------------------------- */
static double orc_fact(int n) { double r = 1.0; for (int i = 2; i <= n; ++i) r *= i; return r; }

void orc_sh(int degree, double x, double y, double z, double* out) {
    const double pi = 3.14159265358979323846;
    double pbar[9][9];
    memset(pbar, 0, sizeof pbar);
    for (int m = 0; m < degree; ++m) {
        double pmm = (m % 2) ? -1.0 : 1.0; /* (-1)^m (2m-1)!! */
        for (int k = 1; k <= 2 * m - 1; k += 2) pmm *= k;
        pbar[m][m] = pmm;
        if (m + 1 < degree) pbar[m + 1][m] = z * (2 * m + 1) * pmm;
        for (int l = m + 2; l < degree; ++l)
            pbar[l][m] = ((2 * l - 1) * z * pbar[l - 1][m] - (l + m - 1) * pbar[l - 2][m]) / (l - m);
    }
    double re[9], im[9];
    re[0] = 1.0; im[0] = 0.0;
    for (int m = 1; m < 9; ++m) {
        re[m] = re[m - 1] * x - im[m - 1] * y;
        im[m] = re[m - 1] * y + im[m - 1] * x;
    }
    for (int l = 0; l < degree; ++l) {
        for (int m = -l; m <= l; ++m) {
            const int am = m < 0 ? -m : m;
            const double K = sqrt((2.0 * l + 1.0) / (4.0 * pi) * orc_fact(l - am) / orc_fact(l + am));
            double v;
            if (m > 0) v = sqrt(2.0) * K * pbar[l][am] * re[am];
            else if (m < 0) v = sqrt(2.0) * K * pbar[l][am] * im[am];
            else v = K * pbar[l][0];
            out[l * l + l + m] = v;
        }
    }
}

/* ---------------------------------------------------------------------------------------------
 * Encoding (composite concatenation, composite.h:215-281)
 * ------------------------------------------------------------------------------------------- */
static void orc_encode_row(const OrcModel* m, const float* row, const double* params, float ml, double* enc) {
    for (int si = 0; si < m->n_slots; ++si) {
        const OrcSlot* s = &m->slots[si];
        double* o = enc + s->out_begin;
        switch (s->type) {
            case ORC_GRID: {
                const OrcGrid* g = &m->grids[s->grid];
                for (int l = 0; l < g->n_levels; ++l) {
                    double f0 = 0.0, f1 = 0.0;
                    if (!orc_masked_fwd(l, ml, g->n_levels)) {
                        uint32_t e[8];
                        double w[8];
                        const int nc = orc_corners(g, l, row + s->in_begin, e, w);
                        const double* tab = params + g->param_offset + 2 * (int64_t)g->offset[l];
                        for (int c = 0; c < nc; ++c) {
                            f0 += w[c] * tab[2 * (int64_t)e[c]];
                            f1 += w[c] * tab[2 * (int64_t)e[c] + 1];
                        }
                    }
                    o[2 * l] = f0;
                    o[2 * l + 1] = f1;
                }
                for (int p = 0; p < s->n_pad; ++p) o[2 * g->n_levels + p] = 0.0;
                break;
            }
            case ORC_SH: {
                for (int p = 0; p < s->n_pad; ++p) o[p] = 1.0;
                const double x = (double)row[s->in_begin] * 2.0 - 1.0;
                const double y = (double)row[s->in_begin + 1] * 2.0 - 1.0;
                const double z = (double)row[s->in_begin + 2] * 2.0 - 1.0;
                orc_sh(s->degree, x, y, z, o + s->n_pad);
                break;
            }
            case ORC_IDENTITY: {
                for (int j = 0; j < s->n_in; ++j) o[j] = (double)row[s->in_begin + j] * s->scale + s->offset;
                for (int p = 0; p < s->n_pad; ++p) o[s->n_in + p] = 1.0;
                break;
            }
            case ORC_ONEHOT: {
                int bin = (int)floorf(row[s->in_begin] * (float)s->n_bins);
                if (bin < 0) bin = 0;
                if (bin >= s->n_bins) bin = s->n_bins - 1;
                for (int j = 0; j < s->n_bins; ++j) o[j] = j == bin ? 1.0 : 0.0;
                for (int p = 0; p < s->n_pad; ++p) o[s->n_bins + p] = 0.0;
                break;
            }
            default: break;
        }
    }
}

void orc_encode(const OrcModel* m, int64_t n, const float* in, const double* params, const float* max_level,
                float max_level_scalar, double* enc) {
    for (int64_t i = 0; i < n; ++i)
        orc_encode_row(m, in + i * m->n_input, params, max_level ? max_level[i] : max_level_scalar, enc + i * m->enc_width);
}

/* ---------------------------------------------------------------------------------------------
 * MLP (fully_fused_mlp.cu): h_{l+1} = act(W_l h_l), output layer padded to 16 rows.
 * ------------------------------------------------------------------------------------------- */
static double orc_act(int act, double v) {
    switch (act) {
        case ORC_ACT_RELU: return v > 0.0 ? v : 0.0;
        case ORC_ACT_SIGMOID: return 1.0 / (1.0 + exp(-v));
        case ORC_ACT_EXP: return exp(v);
        default: return v;
    }
}
static double orc_act_grad_out(int act, double y) {
    switch (act) {
        case ORC_ACT_RELU: return y > 0.0 ? 1.0 : 0.0;
        case ORC_ACT_SIGMOID: return y * (1.0 - y);
        case ORC_ACT_EXP: return y;
        default: return 1.0;
    }
}

/* acts: buffer of (n_layers) * 256 doubles: acts[l] = input of layer l (acts[0] = encoding). */
static void orc_mlp_row(const OrcModel* m, const double* params, const double* enc, double* acts, double* y16) {
    memcpy(acts, enc, sizeof(double) * m->enc_width);
    for (int l = 0; l < m->n_layers; ++l) {
        const double* W = params + m->layer_offset[l];
        const double* a = acts + 256 * l;
        const int nin = m->layer_in[l], nout = m->layer_out[l];
        const int last = l + 1 == m->n_layers;
        double* o = last ? y16 : acts + 256 * (l + 1);
        for (int j = 0; j < nout; ++j) {
            double s = 0.0;
            for (int k = 0; k < nin; ++k) s += W[(int64_t)j * nin + k] * a[k];
            o[j] = orc_act(last ? m->out_act : m->act, s);
        }
    }
}

void orc_forward(const OrcModel* m, int64_t n, const float* in, const double* params, const float* max_level,
                 float max_level_scalar, double* out, double* y16) {
#pragma omp parallel
    {
        double* enc = (double*)malloc(sizeof(double) * 256);
        double* acts = (double*)malloc(sizeof(double) * 256 * ORC_MAX_LAYERS);
        double y[16];
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            orc_encode_row(m, in + i * m->n_input, params, max_level ? max_level[i] : max_level_scalar, enc);
            orc_mlp_row(m, params, enc, acts, y);
            if (out)
                for (int c = 0; c < m->n_output; ++c) out[i * m->n_output + c] = y[c];
            if (y16) memcpy(y16 + i * 16, y, sizeof y);
        }
        free(enc);
        free(acts);
    }
}

/* losses/*.h: value / n_total, gradient * loss_scale / n_total, then output activation derivative. */
void orc_loss(const OrcModel* m, int loss_kind, int64_t n, const double* y16, const float* target, double loss_scale,
              double* loss, double* dz16) {
    const double n_total = (double)n * (double)m->n_output;
    double total = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        for (int c = 0; c < 16; ++c) {
            double g = 0.0;
            if (c < m->n_output) {
                const double y = y16[i * 16 + c];
                const double t = target[i * m->n_output + c];
                double v;
                if (loss_kind == ORC_LOSS_BCE) {
                    const double eps = (double)1e-5f;
                    double p = y < eps ? eps : y;
                    if (p > 1.0 - eps) p = 1.0 - eps;
                    v = -(t * log(p) + (1.0 - t) * log(1.0 - p));
                    g = -(t - p) / (p - p * p);
                } else if (loss_kind == ORC_LOSS_RELL2) {
                    const double den = y * y + (double)0.01f;
                    v = (y - t) * (y - t) / den;
                    g = 2.0 * (y - t) / den;
                } else {
                    v = (y - t) * (y - t);
                    g = 2.0 * (y - t);
                }
                total += v / n_total;
                g = g * loss_scale / n_total * orc_act_grad_out(m->out_act, y);
            }
            if (dz16) dz16[i * 16 + c] = g;
        }
    }
    if (loss) *loss = total;
}

void orc_backward(const OrcModel* m, int64_t n, const float* in, const double* params, const float* max_level,
                  float max_level_scalar, const double* dz16, double* grads) {
    double* enc = (double*)malloc(sizeof(double) * 256);
    double* acts = (double*)malloc(sizeof(double) * 256 * ORC_MAX_LAYERS);
    double* delta = (double*)malloc(sizeof(double) * 256);
    double* nd = (double*)malloc(sizeof(double) * 256);
    double y[16];
    for (int64_t i = 0; i < n; ++i) {
        const float* row = in + i * m->n_input;
        const float ml = max_level ? max_level[i] : max_level_scalar;
        orc_encode_row(m, row, params, ml, enc);
        orc_mlp_row(m, params, enc, acts, y);
        for (int c = 0; c < 16; ++c) delta[c] = dz16[i * 16 + c];
        for (int l = m->n_layers - 1; l >= 0; --l) {
            const double* W = params + m->layer_offset[l];
            double* G = grads + m->layer_offset[l];
            const double* a = acts + 256 * l;
            const int nin = m->layer_in[l], nout = m->layer_out[l];
            for (int o = 0; o < nout; ++o) {
                if (delta[o] == 0.0) continue;
                for (int k = 0; k < nin; ++k) G[(int64_t)o * nin + k] += delta[o] * a[k];
            }
            for (int k = 0; k < nin; ++k) {
                double s = 0.0;
                for (int o = 0; o < nout; ++o) s += delta[o] * W[(int64_t)o * nin + k];
                if (l > 0) s *= (m->act == ORC_ACT_RELU) ? (a[k] > 0.0 ? 1.0 : 0.0) : 1.0;
                nd[k] = s;
            }
            memcpy(delta, nd, sizeof(double) * nin);
        }
        /* delta now holds dL/d(encoding); scatter into grid tables (grid.h:394-517). */
        for (int si = 0; si < m->n_slots; ++si) {
            const OrcSlot* s = &m->slots[si];
            if (s->type != ORC_GRID) continue;
            const OrcGrid* g = &m->grids[s->grid];
            for (int l = 0; l < g->n_levels; ++l) {
                if (orc_skipped_bwd(l, ml, g->n_levels)) continue;
                uint32_t e[8];
                double w[8];
                const int nc = orc_corners(g, l, row + s->in_begin, e, w);
                double* tab = grads + g->param_offset + 2 * (int64_t)g->offset[l];
                const double d0 = delta[s->out_begin + 2 * l], d1 = delta[s->out_begin + 2 * l + 1];
                for (int c = 0; c < nc; ++c) {
                    tab[2 * (int64_t)e[c]] += w[c] * d0;
                    tab[2 * (int64_t)e[c] + 1] += w[c] * d1;
                }
            }
        }
    }
    free(enc);
    free(acts);
    free(delta);
    free(nd);
}

/* adam.h:47-119 in FP32, followed by the EMA update of ema.h:45-76 when ema != NULL. */
void orc_adam_step(const OrcAdam* a, int64_t n_params, int64_t n_matrix, float* params, const float* grads,
                   float* m1, float* m2, uint32_t* steps, float* ema, float ema_decay, float ema_debias_old,
                   float ema_debias_new) {
    for (int64_t i = 0; i < n_params; ++i) {
        const int matrix = i < n_matrix;
        float w = params[i];
        float g = grads[i] / a->loss_scale;
        int skip = matrix ? !a->optimize_matrix : (!a->optimize_non_matrix || g == 0.0f);
        if (!skip) {
            if (matrix) g += a->l2_reg * w;
            const float g2 = g * g;
            m1[i] = a->beta1 * m1[i] + (1.0f - a->beta1) * g;
            m2[i] = a->beta2 * m2[i] + (1.0f - a->beta2) * g2;
            float lr = a->lr;
            if (!matrix) lr *= a->non_matrix_lr_factor;
            const uint32_t step = ++steps[i];
            lr *= sqrtf(1.0f - powf(a->beta2, (float)step)) / (1.0f - powf(a->beta1, (float)step));
            float eff = lr / (sqrtf(m2[i]) + a->eps);
            if (eff < a->lower_lr_bound) eff = a->lower_lr_bound;
            if (eff > a->upper_lr_bound) eff = a->upper_lr_bound;
            const float rel = a->rel_decay * lr, absd = a->abs_decay * lr;
            const float decayed = (1.0f - rel) * w - copysignf(absd, w);
            float nw = decayed - eff * m1[i];
            if (a->clip != 0.0f) nw = nw < -a->clip ? -a->clip : (nw > a->clip ? a->clip : nw);
            params[i] = nw;
            w = nw;
        }
        if (ema) ema[i] = (ema[i] * ema_decay * ema_debias_old + w * (1.0f - ema_decay)) * ema_debias_new;
    }
}

/* ---------------------------------------------------------------------------------------------
 * FP32 scalar forward over all host threads (CPU baseline).
 * ------------------------------------------------------------------------------------------- */
static float orc_actf(int act, float v) {
    switch (act) {
        case ORC_ACT_RELU: return v > 0.f ? v : 0.f;
        case ORC_ACT_SIGMOID: return 1.0f / (1.0f + expf(-v));
        case ORC_ACT_EXP: return expf(v);
        default: return v;
    }
}

int orc_forward_f32(const OrcModel* m, int64_t n, const float* in, const float* params, const float* max_level,
                    float max_level_scalar, float* out, int n_threads) {
    int used = 1;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel
    {
#ifdef _OPENMP
#pragma omp single
        used = omp_get_num_threads();
#endif
        float a[256], b[256];
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            const float* row = in + i * m->n_input;
            const float ml = max_level ? max_level[i] : max_level_scalar;
            for (int si = 0; si < m->n_slots; ++si) {
                const OrcSlot* s = &m->slots[si];
                float* o = a + s->out_begin;
                if (s->type == ORC_GRID) {
                    const OrcGrid* g = &m->grids[s->grid];
                    for (int l = 0; l < g->n_levels; ++l) {
                        float f0 = 0.f, f1 = 0.f;
                        if (!orc_masked_fwd(l, ml, g->n_levels)) {
                            float frac[3];
                            uint32_t cell[3];
                            for (int d = 0; d < 3; ++d) orc_pos_fract(row[s->in_begin + d], g->scale[l], &frac[d], &cell[d]);
                            const float* tab = params + g->param_offset + 2 * (int64_t)g->offset[l];
                            for (int c = 0; c < 8; ++c) {
                                uint32_t q[3];
                                float w = 1.f;
                                for (int d = 0; d < 3; ++d) {
                                    if (c & (1 << d)) { w *= frac[d]; q[d] = cell[d] + 1u; }
                                    else { w *= 1.f - frac[d]; q[d] = cell[d]; }
                                }
                                const uint32_t e = orc_grid_index(g, l, q);
                                f0 += w * tab[2 * (int64_t)e];
                                f1 += w * tab[2 * (int64_t)e + 1];
                            }
                        }
                        o[2 * l] = f0;
                        o[2 * l + 1] = f1;
                    }
                    for (int p = 0; p < s->n_pad; ++p) o[2 * g->n_levels + p] = 0.f;
                } else if (s->type == ORC_SH) {
                    double tmp[64];
                    for (int p = 0; p < s->n_pad; ++p) o[p] = 1.f;
                    orc_sh(s->degree, row[s->in_begin] * 2.f - 1.f, row[s->in_begin + 1] * 2.f - 1.f, row[s->in_begin + 2] * 2.f - 1.f, tmp);
                    for (int j = 0; j < s->degree * s->degree; ++j) o[s->n_pad + j] = (float)tmp[j];
                } else if (s->type == ORC_IDENTITY) {
                    for (int j = 0; j < s->n_in; ++j) o[j] = row[s->in_begin + j] * s->scale + s->offset;
                    for (int p = 0; p < s->n_pad; ++p) o[s->n_in + p] = 1.f;
                } else {
                    int bin = (int)floorf(row[s->in_begin] * (float)s->n_bins);
                    if (bin < 0) bin = 0;
                    if (bin >= s->n_bins) bin = s->n_bins - 1;
                    for (int j = 0; j < s->n_bins; ++j) o[j] = j == bin ? 1.f : 0.f;
                    for (int p = 0; p < s->n_pad; ++p) o[s->n_bins + p] = 0.f;
                }
            }
            float* cur = a;
            float* nxt = b;
            for (int l = 0; l < m->n_layers; ++l) {
                const float* W = params + m->layer_offset[l];
                const int nin = m->layer_in[l], nout = m->layer_out[l];
                const int last = l + 1 == m->n_layers;
                for (int j = 0; j < nout; ++j) {
                    float s = 0.f;
                    for (int k = 0; k < nin; ++k) s += W[(int64_t)j * nin + k] * cur[k];
                    nxt[j] = orc_actf(last ? m->out_act : m->act, s);
                }
                float* t = cur;
                cur = nxt;
                nxt = t;
            }
            for (int c = 0; c < m->n_output; ++c) out[i * m->n_output + c] = cur[c];
        }
    }
    return used;
}

/* ---------------------------------------------------------------------------------------------
 * LoD occupancy pyramid + first active voxel along a ray (see nlod_oracle.h for the sources).
 * IEEE single precision, one rounding per operation (built with -ffp-contract=off); the ray is
 * evaluated with fmaf like nanovdb::Ray::operator().
 * ------------------------------------------------------------------------------------------- */
#include <float.h>

static int orc_bit(const uint32_t* bits, int64_t idx) { return (bits[idx >> 5] >> (31 - (idx & 31))) & 1u; }

void orc_lod_level(const uint32_t* bits0, int32_t res0, int32_t lod, uint32_t* bits_out, uint8_t* leaf_out,
                   uint8_t* lower_out, OrcLodLevel* level) {
    const int32_t r = res0 >> lod;
    const int64_t n = (int64_t)r * r * r;
    const int32_t nb = (r + 7) / 8, nl = (r + 127) / 128;
    memset(bits_out, 0, sizeof(uint32_t) * (size_t)((n + 31) / 32));
    memset(leaf_out, 0, (size_t)nb * nb * nb);
    memset(lower_out, 0, (size_t)nl * nl * nl);
    int32_t bmin[3] = {r, r, r}, bmax[3] = {-1, -1, -1};
    int32_t count = 0;
    const int64_t n0 = (int64_t)res0 * res0 * res0;
    for (int64_t i = 0; i < n0; ++i) {
        if (!orc_bit(bits0, i)) continue;
        const int32_t x = (int32_t)(i % res0) >> lod, y = (int32_t)((i / res0) % res0) >> lod, z = (int32_t)(i / ((int64_t)res0 * res0)) >> lod;
        const int64_t j = x + (int64_t)r * (y + (int64_t)r * z);
        if (!orc_bit(bits_out, j)) {
            bits_out[j >> 5] |= 1u << (31 - (j & 31));
            ++count;
        }
        leaf_out[(x >> 3) + nb * ((y >> 3) + nb * (z >> 3))] = 1;
        lower_out[(x >> 7) + nl * ((y >> 7) + nl * (z >> 7))] = 1;
        const int32_t c[3] = {x, y, z};
        for (int k = 0; k < 3; ++k) {
            if (c[k] < bmin[k]) bmin[k] = c[k];
            if (c[k] > bmax[k]) bmax[k] = c[k];
        }
    }
    level->res = r;
    level->n_active = count;
    for (int k = 0; k < 3; ++k) { level->bbox_min[k] = bmin[k]; level->bbox_max[k] = bmax[k]; }
    level->bits = bits_out;
    level->leaf = leaf_out;
    level->lower = lower_out;
}

/* getDim of a NanoVDB tree holding exactly the active voxels of `L` (one upper node at the origin):
 * 4096 outside it, 128 where no lower node exists, 8 where no leaf exists, 1 inside a leaf. */
static int orc_get_dim(const OrcLodLevel* L, const int32_t ijk[3]) {
    if (L->n_active == 0) return 4096;
    for (int k = 0; k < 3; ++k)
        if (ijk[k] < 0 || ijk[k] >= 4096) return 4096;
    const int32_t nl = (L->res + 127) / 128, nb = (L->res + 7) / 8;
    const int32_t lx = ijk[0] >> 7, ly = ijk[1] >> 7, lz = ijk[2] >> 7;
    if (lx >= nl || ly >= nl || lz >= nl || !L->lower[lx + nl * (ly + nl * lz)]) return 128;
    const int32_t bx = ijk[0] >> 3, by = ijk[1] >> 3, bz = ijk[2] >> 3;
    if (bx >= nb || by >= nb || bz >= nb || !L->leaf[bx + nb * (by + nb * bz)]) return 8;
    return 1;
}

typedef struct {
    int32_t dim;
    float t0, t1;
    int32_t voxel[3], step[3];
    float delta[3], next[3];
} OrcHdda;

static void orc_ray_at(const float E[3], const float D[3], float t, float p[3]) {
    for (int k = 0; k < 3; ++k) p[k] = fmaf(t, D[k], E[k]);
}

static void orc_hdda_init(OrcHdda* h, const float E[3], const float D[3], const float inv[3], float t0, float t1, int32_t dim) {
    h->dim = dim;
    h->t0 = t0;
    h->t1 = t1;
    float pos[3];
    orc_ray_at(E, D, t0, pos);
    for (int a = 0; a < 3; ++a) {
        h->voxel[a] = ((int32_t)floorf(pos[a])) & ~(dim - 1);
        h->delta[a] = 0.f;
        if (D[a] == 0.f) {
            h->next[a] = FLT_MAX;
            h->step[a] = 0;
        } else if (inv[a] > 0.f) {
            h->step[a] = 1;
            h->next[a] = t0 + ((float)(h->voxel[a] + dim) - pos[a]) * inv[a];
            h->delta[a] = inv[a];
        } else {
            h->step[a] = -1;
            h->next[a] = t0 + ((float)h->voxel[a] - pos[a]) * inv[a];
            h->delta[a] = -inv[a];
        }
    }
}

static void orc_hdda_update(OrcHdda* h, const float E[3], const float D[3], const float inv[3], int32_t dim) {
    if (h->dim == dim) return;
    h->dim = dim;
    float pos[3];
    orc_ray_at(E, D, h->t0, pos);
    for (int a = 0; a < 3; ++a) {
        h->voxel[a] = ((int32_t)floorf(pos[a])) & ~(dim - 1);
        if (h->step[a] == 0) continue;
        h->next[a] = h->t0 + ((float)h->voxel[a] - pos[a]) * inv[a];
        if (h->step[a] > 0) h->next[a] += (float)dim * inv[a];
    }
}

static int orc_hdda_step(OrcHdda* h) {
    const float* v = h->next;
    const int a = (v[0] < v[1] && v[0] < v[2]) ? 0 : (v[1] < v[2] ? 1 : 2);
    if (h->next[a] <= h->t0) h->next[a] += h->t0 - 0.999999f * h->next[a] + 1.0e-6f;
    h->t0 = h->next[a];
    h->next[a] += (float)h->dim * h->delta[a];
    h->voxel[a] += h->dim * h->step[a];
    return h->t0 <= h->t1;
}

static int orc_slab(const float o[3], const float d[3], const int32_t ijk[3], float* near_t, float* far_t) {
    *near_t = -1e20f;
    *far_t = 1e20f;
    for (int i = 0; i < 3; ++i) {
        const float inv = 1.f / d[i];
        const float lo = (float)ijk[i], hi = lo + 1.0f;
        if (d[i] == 0.f) {
            if (o[i] < lo || o[i] > hi) return 0;
        } else {
            float t1 = (lo - o[i]) * inv, t2 = (hi - o[i]) * inv;
            if (t1 > t2) { const float t = t1; t1 = t2; t2 = t; }
            *near_t = (t1 < *near_t) ? *near_t : t1;
            *far_t = (*far_t < t2) ? *far_t : t2;
            if (!(*near_t < *far_t) || (double)*far_t < 0.0) return 0;
        }
    }
    return 1;
}

int orc_first_active_voxel(const OrcLodLevel* L, const float E[3], const float D[3], float t_min, const int32_t prev[3],
                           int32_t ijk_out[3], float* t_near, float* t_far) {
    return orc_first_active_voxel_clip(L, E, D, t_min, FLT_MAX, prev, ijk_out, t_near, t_far);
}

int orc_first_active_voxel_clip(const OrcLodLevel* L, const float E[3], const float D[3], float t_min, float t_max,
                                const int32_t prev[3], int32_t ijk_out[3], float* t_near, float* t_far) {
    if (L->n_active == 0) return 0;
    const float inv[3] = {1.f / D[0], 1.f / D[1], 1.f / D[2]};
    /* Ray::clip against the root bbox [min, max + 1), within [t_min, t_max] */
    float t0 = t_min, t1 = t_max;
    for (int i = 0; i < 3; ++i) {
        float a = (float)L->bbox_min[i], b = (float)(L->bbox_max[i] + 1);
        if (a >= b) return 0;
        a = (a - E[i]) * inv[i];
        b = (b - E[i]) * inv[i];
        if (a > b) { const float t = a; a = b; b = t; }
        if (a > t0) t0 = a;
        if (b < t1) t1 = b;
        if (t0 > t1) return 0;
    }
    /* TreeMarcher::init */
    const float ta = t0 + 0.000001f, tb = t1 - 0.000001f;
    if (ta > tb) return 0;
    int32_t ijk[3], leaf[3] = {0, 0, 0};
    int have_leaf = 0;
    float p[3];
    orc_ray_at(E, D, ta, p);
    for (int k = 0; k < 3; ++k) ijk[k] = (int32_t)floorf(p[k]);
    int dim = orc_get_dim(L, ijk);
    if (dim == 1) { have_leaf = 1; for (int k = 0; k < 3; ++k) leaf[k] = ijk[k] >> 3; }
    OrcHdda h;
    orc_hdda_init(&h, E, D, inv, ta, tb, dim > 8 ? dim : 8);
    float mt0 = dim <= 1 ? h.t0 : -1.f;
    const float tmax = tb;
    /* TreeMarcher::step loop with the per-leaf DDA search */
    int valid;
    do {
        const float s0 = mt0;
        const int cur_have = have_leaf;
        const int32_t cur[3] = {leaf[0], leaf[1], leaf[2]};
        valid = orc_hdda_step(&h);
        orc_ray_at(E, D, h.t0 + 0.01f, p);
        int32_t nxt[3];
        for (int k = 0; k < 3; ++k) nxt[k] = (int32_t)floorf(p[k]);
        const int nd = orc_get_dim(L, nxt);
        if (nd == 1) { have_leaf = 1; for (int k = 0; k < 3; ++k) leaf[k] = nxt[k] >> 3; }
        orc_hdda_update(&h, E, D, inv, nd > 8 ? nd : 8);
        mt0 = nd <= 1 ? h.t0 : -1.f;
        if (s0 >= 0.f) {
            const float s1 = (tmax < h.t0) ? tmax : h.t0;
            if (s0 >= s1 || !cur_have) continue;
            OrcHdda dda;
            orc_hdda_init(&dda, E, D, inv, s0, s1, 1);
            do {
                const int32_t* v = dda.voxel;
                if (v[0] - cur[0] * 8 < 0 || v[1] - cur[1] * 8 < 0 || v[2] - cur[2] * 8 < 0 || v[0] - cur[0] * 8 >= 8 ||
                    v[1] - cur[1] * 8 >= 8 || v[2] - cur[2] * 8 >= 8)
                    continue;
                if (v[0] >= L->res || v[1] >= L->res || v[2] >= L->res) continue;
                if (!orc_bit(L->bits, v[0] + (int64_t)L->res * (v[1] + (int64_t)L->res * v[2]))) continue;
                if (v[0] == prev[0] && v[1] == prev[1] && v[2] == prev[2]) continue;
                if (orc_slab(E, D, v, t_near, t_far)) {
                    for (int k = 0; k < 3; ++k) ijk_out[k] = v[k];
                    return 1;
                }
            } while (orc_hdda_step(&dda));
        }
    } while (valid);
    return 0;
}

/* ---------------------------------------------------------------------------------------------
 * Conservative surface voxelization (restating neural_lod/cuda_voxelizer/src/voxelize.cu:58-190,
 * the kernel the reference pipeline runs; cpu_voxelizer.cpp:39-190 is the same test) with glm
 * 0.9.9.8's expressions: dot = (a.x*b.x + a.y*b.y) + a.z*b.z, cross = (a.y*b.z - b.y*a.z, ...),
 * normalize(v) = v * (1 / sqrt(dot(v, v))), min/max/clamp by comparison; and with the fused
 * multiply-adds of the reference kernel as nvcc builds it by default (the reference's CMake passes
 * no -fmad flag).  Which products nvcc fuses was established by running that build, compiled from
 * its source, against candidate restatements (bit for bit on 4.8 M voxels of random triangle
 * soups at 100^3, 256^3 and 512^3, and on the 82.4 M voxels of the 2.0 M-triangle scene at 1024^3):
 *   per triangle  cross: fma(a.y, b.z, -(b.y*a.z)) ...; dot3: fma(a.z, b.z, fma(a.x, b.x, a.y*b.y));
 *                 edge offsets: -1 * fma(n1, v_b, n0*v_a) (the product of the edge vector's negated
 *                 component is the one left unfused)
 *   per voxel     n.p: fma(n.x, p.x, n.y*p.y) + n.z*p.z (the products invariant over the innermost
 *                 x loop are computed apart), except (n.x*p.x + n.y*p.y) + n.z*p.z in the first
 *                 voxel of a row with an odd voxel count (the x loop is unrolled by two and that
 *                 voxel runs on its own); XY and YZ edge tests: fma(n0, p_a, n1*p_b) + d;
 *                 ZX edge tests: fma(n1, p.x, n0*p.z) + d.
 * Every other operation is rounded once (built with -ffp-contract=off; fmaf rounds once).
 * ------------------------------------------------------------------------------------------- */
static float orc_fmin(float a, float b) { return (b < a) ? b : a; }
static float orc_fmax(float a, float b) { return (a < b) ? b : a; }
static float orc_dot3(const float a[3], const float b[3]) { return fmaf(a[2], b[2], fmaf(a[0], b[0], a[1] * b[1])); }

/* createMeshBBCube (util.h:87-112): cube around the mesh bbox, padded by epsilon * extent. */
void orc_mesh_frame(const float mn[3], const float mx[3], uint32_t grid, float eps, float bmin[3], float bmax[3], float unit[3]) {
    float len[3];
    for (int i = 0; i < 3; ++i) len[i] = mx[i] - mn[i];
    const float ml = orc_fmax(len[0], orc_fmax(len[1], len[2]));
    for (int i = 0; i < 3; ++i) {
        bmin[i] = mn[i];
        bmax[i] = mx[i];
        if (ml == len[i]) continue;
        const float delta = ml - len[i];
        bmin[i] = mn[i] - delta / 2.0f;
        bmax[i] = mx[i] + delta / 2.0f;
    }
    if (eps != 0.f) {
        float e[3];
        for (int i = 0; i < 3; ++i) e[i] = (bmax[i] - bmin[i]) * eps;
        for (int i = 0; i < 3; ++i) { bmin[i] -= e[i]; bmax[i] += e[i]; }
    }
    for (int i = 0; i < 3; ++i) unit[i] = (bmax[i] - bmin[i]) / (float)grid;   /* voxinfo, util.h:58-63 */
}

void orc_voxelize(const float* tris, int64_t n, const float bmin[3], const float unit[3], uint32_t grid, uint32_t* bits) {
    const float gmax = (float)(grid - 1);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < n; ++t) {
        const float* T = tris + 9 * t;
        float v0[3], v1[3], v2[3], e0[3], e1[3], e2[3], cr[3], nrm[3];
        for (int i = 0; i < 3; ++i) { v0[i] = T[i] - bmin[i]; v1[i] = T[3 + i] - bmin[i]; v2[i] = T[6 + i] - bmin[i]; }
        for (int i = 0; i < 3; ++i) { e0[i] = v1[i] - v0[i]; e1[i] = v2[i] - v1[i]; e2[i] = v0[i] - v2[i]; }
        cr[0] = fmaf(e0[1], e1[2], -(e1[1] * e0[2]));
        cr[1] = fmaf(e0[2], e1[0], -(e1[2] * e0[0]));
        cr[2] = fmaf(e0[0], e1[1], -(e1[0] * e0[1]));
        const float inv_len = 1.0f / sqrtf(orc_dot3(cr, cr));
        for (int i = 0; i < 3; ++i) nrm[i] = cr[i] * inv_len;
        int32_t lo[3], hi[3];
        for (int i = 0; i < 3; ++i) {
            const float wmin = orc_fmin(v0[i], orc_fmin(v1[i], v2[i])), wmax = orc_fmax(v0[i], orc_fmax(v1[i], v2[i]));
            lo[i] = (int32_t)orc_fmin(orc_fmax(wmin / unit[i], 0.0f), gmax);
            hi[i] = (int32_t)orc_fmin(orc_fmax(wmax / unit[i], 0.0f), gmax);
        }
        float c[3] = {0.f, 0.f, 0.f};
        for (int i = 0; i < 3; ++i)
            if (nrm[i] > 0.0f) c[i] = unit[i];
        float cv[3], dc[3];
        for (int i = 0; i < 3; ++i) { cv[i] = c[i] - v0[i]; dc[i] = (unit[i] - c[i]) - v0[i]; }
        const float d1 = orc_dot3(nrm, cv), d2 = orc_dot3(nrm, dc);
        /* edge normals in the XY, YZ and ZX planes and their offsets (axis a, axis b) */
        const int ax[3][2] = {{0, 1}, {1, 2}, {2, 0}};
        const int flip_axis[3] = {2, 0, 1};
        const float* E[3] = {e0, e1, e2};
        const float* V[3] = {v0, v1, v2};
        float ne[3][3][2], de[3][3];
        for (int pl = 0; pl < 3; ++pl) {
            const int a = ax[pl][0], b = ax[pl][1];
            for (int k = 0; k < 3; ++k) {
                float n0 = -1.0f * E[k][b], n1 = E[k][a];
                if (nrm[flip_axis[pl]] < 0.0f) { n0 = -n0; n1 = -n1; }
                ne[pl][k][0] = n0;
                ne[pl][k][1] = n1;
                de[pl][k] = ((-1.0f * fmaf(n1, V[k][b], n0 * V[k][a])) + orc_fmax(0.0f, unit[a] * n0)) + orc_fmax(0.0f, unit[b] * n1);
            }
        }
        for (int z = lo[2]; z <= hi[2]; ++z)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int x = lo[0]; x <= hi[0]; ++x) {
                    const float p[3] = {(float)x * unit[0], (float)y * unit[1], (float)z * unit[2]};
                    /* the reference build fuses n.x * p.x into the plane dot product, except in the
                       first voxel of a row with an odd voxel count: its loop over x runs in pairs
                       after that one, which rounds all three products */
                    float nd;
                    if (x == lo[0] && ((hi[0] - lo[0]) & 1) == 0) {
                        const float px = nrm[0] * p[0], py = nrm[1] * p[1], pz = nrm[2] * p[2];
                        nd = (px + py) + pz;
                    } else {
                        nd = fmaf(nrm[0], p[0], nrm[1] * p[1]) + nrm[2] * p[2];
                    }
                    if ((nd + d1) * (nd + d2) > 0.0f) continue;
                    int ok = 1;
                    for (int pl = 0; pl < 3 && ok; ++pl) {
                        const int a = ax[pl][0], b = ax[pl][1];
                        for (int k = 0; k < 3; ++k) {
                            const float n0 = ne[pl][k][0], n1 = ne[pl][k][1];
                            const float s = pl == 2 ? fmaf(n1, p[b], n0 * p[a]) : fmaf(n0, p[a], n1 * p[b]);
                            if (s + de[pl][k] < 0.0f) { ok = 0; break; }
                        }
                    }
                    if (!ok) continue;
                    const uint64_t loc = (uint64_t)x + (uint64_t)y * grid + (uint64_t)z * grid * grid;
#pragma omp atomic
                    bits[loc >> 5] |= 1u << (31 - (loc & 31));
                }
    }
}

void orc_first_active_voxel_batch(const OrcLodLevel* L, int64_t n, const float* eye, const float* dir, const float* t_min,
                                  const int32_t* prev, int32_t* hit, int32_t* ijk, float* t_near, float* t_far) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        const int32_t none[3] = {-1, -1, -1};
        float tn = 0.f, tf = 0.f;
        int32_t v[3] = {0, 0, 0};
        hit[i] = orc_first_active_voxel(L, eye + 3 * i, dir + 3 * i, t_min ? t_min[i] : 0.f, prev ? prev + 3 * i : none, v, &tn, &tf);
        for (int k = 0; k < 3; ++k) ijk[3 * i + k] = hit[i] ? v[k] : 0;
        t_near[i] = hit[i] ? tn : 0.f;
        t_far[i] = hit[i] ? tf : 0.f;
    }
}

/* ---------------------------------------------------------------------------------------------
 * Wavefront render query, one ray at a time (restating the renderer of this library, which
 * follows rptr/cuda/neural-lod/wavefront_neural_throughput_visibility_lod.cu:470-720 and the
 * per-ray steps of rptr/cuda/wavefront_neural_pt.cuh).  Geometry and sampling in IEEE single
 * precision without contraction (bit-identical rays), networks in FP64 through orc_forward.
 * ------------------------------------------------------------------------------------------- */
static uint32_t orc_mix32(uint32_t h) {
    h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
    return h;
}
static float orc_u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }

static void orc_sample_sphere(uint32_t key, float w[3]) {
    for (uint32_t t = 0; t < 16; ++t) {
        const uint32_t h = orc_mix32(key + t * 0x632BE5ABu);
        const float x = 2.f * orc_u01(h) - 1.f;
        const float y = 2.f * orc_u01(orc_mix32(h ^ 0x68E31DA4u)) - 1.f;
        const float z = 2.f * orc_u01(orc_mix32(h ^ 0xB5297A4Du)) - 1.f;
        const float r2 = (x * x + y * y) + z * z;
        if (r2 <= 1.f && r2 >= 1e-4f) {
            const float r = sqrtf(r2);
            w[0] = x / r; w[1] = y / r; w[2] = z / r;
            return;
        }
    }
    w[0] = 0.f; w[1] = 0.f; w[2] = 1.f;
}

void orc_render(const OrcModel* vis, const double* vis_params, const OrcModel* thr, const double* thr_params, const OrcLodLevel* L,
                const OrcRenderParams* p, const float cam[12], float* image, uint32_t* ray_stats, uint64_t* totals) {
    const int64_t n = (int64_t)p->width * p->height;
    const uint32_t seed_lo = (uint32_t)p->seed, seed_hi = (uint32_t)(p->seed >> 32);
    const float res = (float)L->res;
    uint64_t tv = 0, tt = 0, dropped = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : tv, tt, dropped)
    for (int64_t ray = 0; ray < n; ++ray) {
        const uint32_t px = (uint32_t)(ray % p->width), py = (uint32_t)(ray / p->width);
        const float W = (float)p->width, H = (float)p->height;
        const float a = (2.f * ((float)px + 0.5f) - W) / W;
        const float b = (H - 2.f * ((float)py + 0.5f)) / H;
        float o[3], d[3], dd[3], tp[3] = {1.f, 1.f, 1.f};
        for (int k = 0; k < 3; ++k) dd[k] = (a * cam[3 + k] + b * cam[6 + k]) + cam[9 + k];
        const float len = sqrtf((dd[0] * dd[0] + dd[1] * dd[1]) + dd[2] * dd[2]);
        for (int k = 0; k < 3; ++k) { o[k] = cam[k]; d[k] = dd[k] / len; }
        int32_t ijk[3] = {-1, -1, -1};
        float tmin = 0.f;
        uint32_t bounce = 0, nvis = 0, qv = 0, qt = 0;
        float* img = image + 3 * ray;
        img[0] = img[1] = img[2] = 0.f;
        for (;;) {
            if (nvis >= p->max_vis) { dropped++; break; }
            int32_t v[3];
            float tn = 0.f, tf = 0.f;
            if (!orc_first_active_voxel(L, o, d, tmin, ijk, v, &tn, &tf)) {
                for (int k = 0; k < 3; ++k) img[k] = bounce == 0 ? p->background[k] : tp[k] * p->env[k];
                break;
            }
            for (int k = 0; k < 3; ++k) ijk[k] = v[k];
            ++nvis;
            ++qv;
            float in[10];
            for (int k = 0; k < 3; ++k) {
                const float pk = o[k] + d[k] * tn;
                float l = pk - (float)ijk[k];
                l = l < 0.f ? 0.f : (l > 1.f ? 1.f : l);
                in[k] = l;
                in[3 + k] = (d[k] + 1.f) * 0.5f;
            }
            double vo;
            orc_forward(vis, 1, in, vis_params, NULL, p->lod_max_level, &vo, NULL);
            if (vo >= (double)p->threshold) {
                if (bounce + 1 >= p->max_depth) break;   /* hit on the last path vertex: dark */
                float wi[3];
                orc_sample_sphere(orc_mix32(orc_mix32((uint32_t)ray ^ orc_mix32(seed_lo ^ orc_mix32(seed_hi))) ^ (bounce * 0x9E3779B9u)), wi);
                for (int k = 0; k < 3; ++k) {
                    in[k] = ((float)ijk[k] + 0.5f) / res;
                    in[3 + k] = (wi[k] + 1.f) * 0.5f;
                    in[6 + k] = (-d[k] + 1.f) * 0.5f;
                }
                in[9] = p->lod_input;
                double to[3];
                orc_forward(thr, 1, in, thr_params, NULL, 1000.f, to, NULL);
                ++qt;
                const float t_eps = tn + 1e-4f * (tf - tn);
                int alive = 0;
                for (int k = 0; k < 3; ++k) {
                    const float tk = (float)to[k];
                    tp[k] = tp[k] * ((tk > 0.f ? tk : 0.f) * 12.566370614359172f);
                    alive |= tp[k] != 0.f;
                    o[k] = o[k] + d[k] * t_eps;
                    d[k] = wi[k];
                }
                tmin = 0.f;
                ++bounce;
                nvis = 0;
                if (!alive) break;
            } else {
                tmin = (tn + tf) * 0.5f;
            }
        }
        if (ray_stats) { ray_stats[2 * ray] = qv; ray_stats[2 * ray + 1] = qt; }
        tv += qv;
        tt += qt;
    }
    if (totals) { totals[0] = tv; totals[1] = tt; totals[2] = dropped; }
}

/* ---------------------------------------------------------------------------------------------
 * Per-voxel threshold optimisation (rptr/cuda/neural-lod/neural_lod_learning.cu:122-293,
 * metrics neural_lod_learning_common.cuh:836-927), float arithmetic without contraction.
 * ------------------------------------------------------------------------------------------- */
static float orc_prec(uint32_t fp, uint32_t tp) { return tp == 0 ? 0.f : (float)tp / (float)(tp + fp); }
static float orc_rec(uint32_t fn, uint32_t tp) { return tp == 0 ? 0.f : (float)tp / (float)(tp + fn); }
static float orc_fscore(uint32_t tn, uint32_t fp, uint32_t fn, uint32_t tp, float beta) {
    const float p = orc_prec(fp, tp), r = orc_rec(fn, tp);
    (void)tn;
    if (p + r == 0.f) return 0.f;
    const float b2 = beta * beta;
    return ((1.f + b2) * p * r) / (b2 * p + r);
}

static float orc_score(int metric, uint32_t tn, uint32_t fp, uint32_t fn, uint32_t tp, uint32_t sp, uint32_t sn, float beta) {
    switch (metric) {
        case 0: return orc_prec(fp, tp);
        case 1: return orc_rec(fn, tp);
        case 2: return orc_fscore(tn, fp, fn, tp, beta);
        case 3: return (orc_fscore(tn, fp, fn, tp, beta) + orc_fscore(tp, fn, fp, tn, beta)) * 0.5f;
        case 4: return (orc_fscore(tn, fp, fn, tp, beta) * sp + orc_fscore(tp, fn, fp, tn, beta) * sn) / (sp + sn);
        case 5: return (orc_fscore(tn, fp, fn, tp, beta) * sp + orc_fscore(tp, fn, fp, tn, 1.f) * sn) / (sp + sn);
        case 6: {
            const float numer = (float)(tp * tn) - (float)(fp * fn);
            const float den = (float)(tp + fp) * (float)(tp + fn) * (float)(tn + fp) * (float)(tn + fn);
            return den == 0 ? 0.f : numer / sqrtf(den);
        }
        case 7: {
            const float numer = 2.f * ((float)(tp * tn) - (float)(fn * fp));
            const float den = (float)(tp + fp) * (float)(fp + tn) + (float)(tp + fn) * (float)(fn + tn);
            return den == 0 ? 0.f : numer / den;
        }
        case 8: {
            const float den = (float)(tp + tn + fp + fn);
            return den == 0 ? 0.f : (float)(tp + tn) / den;
        }
        case 9: {
            const float se = tp == 0 ? 0.0f : (float)tp / (float)(tp + fn), spc = tn == 0 ? 0.0f : (float)tn / (float)(tn + fp);
            return (se + spc) * 0.5f;
        }
        case 10: return sqrtf(orc_prec(fp, tp) * orc_rec(fn, tp));
        case 11: {
            const float se = tp == 0 ? 0.0f : (float)tp / (float)(tp + fn), spc = tn == 0 ? 0.0f : (float)tn / (float)(tn + fp);
            return se + spc - 1.f;
        }
        default: return 0.f;
    }
}

void orc_optimal_thresholds(const float* truth, const float* proba, uint32_t n_samples, uint32_t n_voxels, int metric, float beta,
                            float* out) {
    enum { T = 101 };
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t v = 0; v < (int64_t)n_voxels; ++v) {
        const float* tr = truth + v * (int64_t)n_samples;
        const float* pr = proba + v * (int64_t)n_samples;
        uint32_t pos = 0;
        for (uint32_t i = 0; i < n_samples; ++i) pos += tr[i] == 1.0f;
        float sc[T];
        for (int k = 0; k < T; ++k) {
            const float th = k / (float)(T - 1);
            uint32_t tn = 0, fp = 0, fn = 0, tp = 0;
            for (uint32_t i = 0; i < n_samples; ++i) {
                const int pred = pr[i] > th, t = tr[i] == 1.0f;
                if (!t) { if (pred) ++fp; else ++tn; }
                else { if (pred) ++tp; else ++fn; }
            }
            sc[k] = orc_score(metric, tn, fp, fn, tp, pos, n_samples - pos, beta);
        }
        float best = -10.0f;
        int opt = 0;
        for (int k = 0; k < T; ++k)
            if (sc[k] > best) { best = sc[k]; opt = k; }
        int eq = 0;
        /* neural_lod_learning.cu:257 compares with the double 1e-4; 1e-4f is the largest float
           below it, so "<= 1e-4f" is the same test */
        while (opt + eq < T && fabsf(sc[opt + eq] - sc[opt]) <= 1e-4f) ++eq;
        opt += eq / 2;
        out[v] = opt / (float)(T - 1);
    }
}
