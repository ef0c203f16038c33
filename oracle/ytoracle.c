/*
 * ytoracle.c -- CPU restatement of yt's grid ray-casting sampler path.
 *
 * TEST INFRASTRUCTURE.  This is the oracle the GPU renderer is checked
 * against; only tests, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py load it.  It is compiled with -ffp-contract=off so that every
 * float64 operation rounds exactly as yt's compiled Cython/C++ does on an
 * x86-64 host (SSE2, no fused multiply-add), on any host.
 *
 * Each function restates one reference routine, keeping its order of
 * floating-point operations (the order decides the last bit):
 *   yo_walk_volume          yt/utilities/lib/grid_traversal.pyx:26-140
 *   yo_offset_interpolate   yt/utilities/lib/fixed_interpolator.cpp:13,34-52
 *   fit_init / fit_get /
 *   fit_eval_transfer       yt/utilities/lib/field_interpolation_tables.pxd:44-110
 *   sample_vr               yt/utilities/lib/image_samplers.pyx:449-487
 *   sample_projection       yt/utilities/lib/image_samplers.pyx:327-343
 *   sample_interp_proj      yt/utilities/lib/image_samplers.pyx:368-403
 *   sample_mip              (no reference: ProjectionSampler with max)
 *   extent_plane_parallel   yt/utilities/lib/lenses.pyx:22-55
 *   extent_perspective      yt/utilities/lib/lenses.pyx:60-161
 *   extent_null             yt/utilities/lib/lenses.pyx:169-175
 *   vector_plane_parallel   yt/utilities/lib/lenses.pyx:179-192
 *   vector_null             yt/utilities/lib/lenses.pyx:196-207
 *   yo_cast_through_kdtree  yt/utilities/lib/image_samplers.pyx:146-197
 *   yo_ghost_zone_interpolate yt/utilities/lib/interpolators.pyx:177-226
 *
 * Additionally yo_trace_* record a per-ray hash of every visited cell
 * (brick, index, enter_t bits, exit_t bits) so that the GPU traversal can be
 * compared bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define YO_VR 0
#define YO_PROJ 1
#define YO_IPROJ 2
#define YO_MIP 3
#define YO_LIGHT 4

typedef struct {
    double left_edge[3];
    double right_edge[3];
    double dds[3];
    double idds[3];
    int dims[3];
    int n_fields;
    const double *data[6];
    const uint8_t *mask;
} yo_vc;

typedef struct {
    const double *values;
    double bounds[2];
    double dbin, idbin;
    double *d0;
    double *dy;
    int field_id, weight_field_id, weight_table_id, nbins;
} yo_fit;

typedef struct {
    int nv[2];
    int lens;      /* 0: plane-parallel vectors, 1: per-pixel vectors */
    int extent;    /* 0: plane-parallel, 1: perspective, 2: null */
    int kind;      /* YO_VR, YO_PROJ, YO_IPROJ, YO_MIP */
    int n_samples;
    int n_fits;
    int grey_opacity;
    int field_table_ids[6];
    const double *vp_pos;  /* plane-parallel: 12 values; else nx*ny*3 */
    const double *vp_dir;  /* plane-parallel: 3 values; else nx*ny*3 */
    double center[3];
    double bounds[4];
    double x_vec[3];
    double y_vec[3];
    double width[3];
    double camera_data[15];
    double pdx, pdy;
    double *image;          /* nx*ny*4 */
    const double *zbuffer;  /* nx*ny */
    yo_fit fits[6];
    double light_dir[3];   /* LightSourceRenderSampler: normalised */
    double light_rgba[4];
} yo_sampler;

/* fp_utils.pxd helpers: first-argument-wins semantics */
static inline double yo_fmax(double a, double b) { if (a > b) return a; return b; }
static inline double yo_fmin(double a, double b) { if (a < b) return a; return b; }
static inline int64_t yo_iclip(int64_t i, int64_t a, int64_t b) { if (i < a) return a; if (i > b) return b; return i; }
static inline double yo_fclip(double f, double a, double b) { return yo_fmin(yo_fmax(f, a), b); }

typedef void (*yo_sample_fn)(const yo_vc *vc, const double v_pos[3], const double v_dir[3],
                             double enter_t, double exit_t, const int index[3], void *data);

int yo_walk_volume(const yo_vc *vc, const double v_pos[3], const double v_dir[3],
                   yo_sample_fn sample, void *data, double *return_t, double max_t)
{
    int cur_ind[3], step[3];
    int x, y, i, hit, direction;
    double intersect_t = 1.1;
    double iv_dir[3] = {0.0, 0.0, 0.0};
    double tmax[3], tdelta[3];
    double exit_t = -1.0, enter_t = -1.0;
    double tl, temp_x, temp_y = -1;
    if (max_t > 1.0) max_t = 1.0;
    direction = -1;
    if (vc->left_edge[0] <= v_pos[0] && v_pos[0] < vc->right_edge[0] &&
        vc->left_edge[1] <= v_pos[1] && v_pos[1] < vc->right_edge[1] &&
        vc->left_edge[2] <= v_pos[2] && v_pos[2] < vc->right_edge[2]) {
        intersect_t = 0.0;
        direction = 3;
    }
    for (i = 0; i < 3; i++) {
        if (v_dir[i] < 0) step[i] = -1;
        else if (v_dir[i] == 0.0) { step[i] = 0; continue; }
        else step[i] = 1;
        iv_dir[i] = 1.0 / v_dir[i];
        if (direction == 3) continue;
        x = (i + 1) % 3;
        y = (i + 2) % 3;
        if (step[i] > 0) tl = (vc->left_edge[i] - v_pos[i]) * iv_dir[i];
        else tl = (vc->right_edge[i] - v_pos[i]) * iv_dir[i];
        temp_x = (v_pos[x] + tl * v_dir[x]);
        temp_y = (v_pos[y] + tl * v_dir[y]);
        if (fabs(temp_x - vc->left_edge[x]) < 1e-10 * vc->dds[x]) temp_x = vc->left_edge[x];
        else if (fabs(temp_x - vc->right_edge[x]) < 1e-10 * vc->dds[x]) temp_x = vc->right_edge[x];
        if (fabs(temp_y - vc->left_edge[y]) < 1e-10 * vc->dds[y]) temp_y = vc->left_edge[y];
        else if (fabs(temp_y - vc->right_edge[y]) < 1e-10 * vc->dds[y]) temp_y = vc->right_edge[y];
        if (vc->left_edge[x] <= temp_x && temp_x <= vc->right_edge[x] &&
            vc->left_edge[y] <= temp_y && temp_y <= vc->right_edge[y] &&
            0.0 <= tl && tl < intersect_t) {
            direction = i;
            intersect_t = tl;
        }
    }
    if (enter_t >= 0.0) intersect_t = enter_t;
    if (!((0.0 <= intersect_t) && (intersect_t < max_t))) return 0;
    for (i = 0; i < 3; i++) {
        tdelta[i] = ((double)step[i] * iv_dir[i]) * vc->dds[i];
        if (i == direction && step[i] > 0) {
            cur_ind[i] = 0;
        } else if (i == direction && step[i] < 0) {
            cur_ind[i] = vc->dims[i] - 1;
        } else {
            temp_x = intersect_t * v_dir[i] + v_pos[i];
            temp_y = ((temp_x - vc->left_edge[i]) * vc->idds[i]);
            if (-1 < temp_y && temp_y < 0 && step[i] > 0) temp_y = 0.0;
            else if (vc->dims[i] - 1 < temp_y && temp_y < vc->dims[i] && step[i] < 0)
                temp_y = vc->dims[i] - 1;
            cur_ind[i] = (int)(floor(temp_y));
        }
        if (step[i] > 0) temp_y = (cur_ind[i] + 1) * vc->dds[i] + vc->left_edge[i];
        else if (step[i] < 0) temp_y = cur_ind[i] * vc->dds[i] + vc->left_edge[i];
        tmax[i] = (temp_y - v_pos[i]) * iv_dir[i];
        if (step[i] == 0) tmax[i] = 1e60;
    }
    for (i = 0; i < 3; i++) {
        if (cur_ind[i] == vc->dims[i] && step[i] >= 0) return 0;
        if (cur_ind[i] == -1 && step[i] <= -1) return 0;
    }
    enter_t = intersect_t;
    hit = 0;
    while (1) {
        hit += 1;
        if (tmax[0] < tmax[1]) {
            if (tmax[0] < tmax[2]) i = 0; else i = 2;
        } else {
            if (tmax[1] < tmax[2]) i = 1; else i = 2;
        }
        exit_t = yo_fmin(tmax[i], max_t);
        sample(vc, v_pos, v_dir, enter_t, exit_t, cur_ind, data);
        cur_ind[i] += step[i];
        enter_t = tmax[i];
        tmax[i] += tdelta[i];
        if (cur_ind[i] < 0 || cur_ind[i] >= vc->dims[i] || enter_t >= max_t) break;
    }
    if (return_t != NULL) return_t[0] = exit_t;
    return hit;
}

double yo_offset_interpolate(const int ds[3], const double dp[3], const double *data)
{
#define OINDEX(A, B, C) data[(A) * (ds[1] + 1) * (ds[2] + 1) + (B) * ds[2] + (B) + (C)]
    double dv, vz[4];
    dv = 1.0 - dp[2];
    vz[0] = dv * OINDEX(0, 0, 0) + dp[2] * OINDEX(0, 0, 1);
    vz[1] = dv * OINDEX(0, 1, 0) + dp[2] * OINDEX(0, 1, 1);
    vz[2] = dv * OINDEX(1, 0, 0) + dp[2] * OINDEX(1, 0, 1);
    vz[3] = dv * OINDEX(1, 1, 0) + dp[2] * OINDEX(1, 1, 1);
    dv = 1.0 - dp[1];
    vz[0] = dv * vz[0] + dp[1] * vz[1];
    vz[1] = dv * vz[2] + dp[1] * vz[3];
    dv = 1.0 - dp[0];
    vz[0] = dv * vz[0] + dp[0] * vz[1];
    return vz[0];
#undef OINDEX
}

/* FIT_initialize_table: d0 / dy are caller-provided buffers of nbins doubles */
void yo_fit_init(yo_fit *fit, int nbins, const double *values, double b1, double b2,
                 int field_id, int weight_field_id, int weight_table_id, double *d0, double *dy)
{
    int i;
    fit->bounds[0] = b1;
    fit->bounds[1] = b2;
    fit->nbins = nbins;
    fit->dbin = (fit->bounds[1] - fit->bounds[0]) / (fit->nbins - 1);
    fit->idbin = 1.0 / fit->dbin;
    fit->values = values;
    fit->d0 = d0;
    fit->dy = dy;
    for (i = 0; i < nbins - 1; i++) {
        fit->d0[i] = fit->bounds[0] + i * fit->dbin;
        fit->dy[i] = (fit->values[i + 1] - fit->values[i]) * fit->idbin;
    }
    fit->field_id = field_id;
    fit->weight_field_id = weight_field_id;
    fit->weight_table_id = weight_table_id;
}

static inline double fit_get(const yo_fit *fit, const double dvs[6])
{
    double dd, dout, v = dvs[fit->field_id];
    int bin_id;
    if (v >= fit->bounds[1] || v <= fit->bounds[0]) return 0.0;
    if (!isnormal(v)) return 0.0;
    bin_id = (int)((v - fit->bounds[0]) * fit->idbin);
    bin_id = (int)yo_iclip(bin_id, 0, fit->nbins - 2);
    dd = v - fit->d0[bin_id];
    dout = fit->values[bin_id] + dd * fit->dy[bin_id];
    if (fit->weight_field_id != -1) dout *= dvs[fit->weight_field_id];
    return dout;
}

static inline void fit_eval_transfer(double dt, const double *dvs, double *rgba, int n_fits,
                                     const yo_fit fits[6], const int field_table_ids[6],
                                     int grey_opacity)
{
    int i, fid;
    double ta;
    double istorage[6] = {0, 0, 0, 0, 0, 0};
    double trgba[6];
    for (i = 0; i < n_fits; i++) istorage[i] = fit_get(&fits[i], dvs);
    for (i = 0; i < n_fits; i++) {
        fid = fits[i].weight_table_id;
        if (fid != -1) istorage[i] *= istorage[fid];
    }
    for (i = 0; i < 6; i++) trgba[i] = istorage[field_table_ids[i]];
    if (grey_opacity == 1) {
        ta = yo_fmax(1.0 - dt * trgba[3], 0.0);
        for (i = 0; i < 4; i++) rgba[i] = dt * trgba[i] + ta * rgba[i];
    } else {
        for (i = 0; i < 3; i++) {
            ta = yo_fmax(1.0 - dt * trgba[i], 0.0);
            rgba[i] = dt * trgba[i] + ta * rgba[i];
        }
    }
}

/* The reference can pass an index outside the brick (an axis with v_dir == 0
 * snapped onto a face from just outside starts at -1, grid_traversal.pyx:67-78
 * and :113-117) and then reads outside its arrays.  Such cells contribute
 * nothing here, as on the GPU. */
static inline int yo_inside(const yo_vc *vc, const int index[3])
{
    return index[0] >= 0 && index[0] < vc->dims[0] && index[1] >= 0 && index[1] < vc->dims[1] &&
           index[2] >= 0 && index[2] < vc->dims[2];
}

typedef struct {
    double rgba[4];
    const yo_sampler *s;
} yo_acc;

static void sample_vr(const yo_vc *vc, const double v_pos[3], const double v_dir[3],
                      double enter_t, double exit_t, const int index[3], void *data)
{
    yo_acc *im = (yo_acc *)data;
    const yo_sampler *s = im->s;
    int i, j, k;
    int offset = index[0] * (vc->dims[1] + 1) * (vc->dims[2] + 1) + index[1] * (vc->dims[2] + 1) + index[2];
    int cell_offset = index[0] * (vc->dims[1]) * (vc->dims[2]) + index[1] * (vc->dims[2]) + index[2];
    double dp[3], ds[3], dt, dvs[6] = {0, 0, 0, 0, 0, 0};
    if (!yo_inside(vc, index)) return;
    if (vc->mask[cell_offset] != 1) return;
    dt = (exit_t - enter_t) / s->n_samples;
    for (i = 0; i < 3; i++) {
        dp[i] = (enter_t + 0.5 * dt) * v_dir[i] + v_pos[i];
        dp[i] -= index[i] * vc->dds[i] + vc->left_edge[i];
        dp[i] *= vc->idds[i];
        ds[i] = v_dir[i] * vc->idds[i] * dt;
    }
    for (k = 0; k < s->n_samples; k++) {
        for (j = 0; j < vc->n_fields; j++) dvs[j] = yo_offset_interpolate(vc->dims, dp, vc->data[j] + offset);
        fit_eval_transfer(dt, dvs, im->rgba, s->n_fits, s->fits, s->field_table_ids, s->grey_opacity);
        for (j = 0; j < 3; j++) dp[j] += ds[j];
    }
}

static void sample_projection(const yo_vc *vc, const double v_pos[3], const double v_dir[3],
                              double enter_t, double exit_t, const int index[3], void *data)
{
    yo_acc *im = (yo_acc *)data;
    int i, n = vc->n_fields < 4 ? vc->n_fields : 4;
    double dl = (exit_t - enter_t);
    int di = (index[0] * vc->dims[1] + index[1]) * vc->dims[2] + index[2];
    (void)v_pos; (void)v_dir;
    if (!yo_inside(vc, index)) return;
    for (i = 0; i < n; i++) im->rgba[i] += vc->data[i][di] * dl;
}

static void sample_mip(const yo_vc *vc, const double v_pos[3], const double v_dir[3],
                       double enter_t, double exit_t, const int index[3], void *data)
{
    yo_acc *im = (yo_acc *)data;
    int i, n = vc->n_fields < 4 ? vc->n_fields : 4;
    int di = (index[0] * vc->dims[1] + index[1]) * vc->dims[2] + index[2];
    (void)v_pos; (void)v_dir; (void)enter_t; (void)exit_t;
    if (!yo_inside(vc, index)) return;
    for (i = 0; i < n; i++) {
        double v = vc->data[i][di];
        if (v > im->rgba[i]) im->rgba[i] = v;
    }
}

static void sample_interp_proj(const yo_vc *vc, const double v_pos[3], const double v_dir[3],
                               double enter_t, double exit_t, const int index[3], void *data)
{
    yo_acc *im = (yo_acc *)data;
    const yo_sampler *s = im->s;
    int i, j, k, n3 = vc->n_fields < 3 ? vc->n_fields : 3;
    int offset = index[0] * (vc->dims[1] + 1) * (vc->dims[2] + 1) + index[1] * (vc->dims[2] + 1) + index[2];
    double dp[3], ds[3], dvs[6] = {0, 0, 0, 0, 0, 0};
    double dt = (exit_t - enter_t) / s->n_samples;
    if (!yo_inside(vc, index)) return;
    for (i = 0; i < 3; i++) {
        dp[i] = (enter_t + 0.5 * dt) * v_dir[i] + v_pos[i];
        dp[i] -= index[i] * vc->dds[i] + vc->left_edge[i];
        dp[i] *= vc->idds[i];
        ds[i] = v_dir[i] * vc->idds[i] * dt;
    }
    for (k = 0; k < s->n_samples; k++) {
        for (j = 0; j < vc->n_fields; j++) dvs[j] = yo_offset_interpolate(vc->dims, dp, vc->data[j] + offset);
        for (j = 0; j < n3; j++) im->rgba[j] += dvs[j] * dt;
        for (j = 0; j < 3; j++) dp[j] += ds[j];
    }
}

/* eval_gradient (fixed_interpolator.cpp:116-148): one-sided or central
 * differences of offset_interpolate, 0.05 apart, normalised to -grad/|grad|. */
static void yo_eval_gradient(const int ds[3], double dp[3], const double *data, double *grad)
{
    int i;
    double denom, plus, minus, backup, normval = 0.0;
    for (i = 0; i < 3; i++) {
        backup = dp[i];
        grad[i] = 0.0;
        if (dp[i] >= 0.95) { plus = dp[i]; minus = dp[i] - 0.05; }
        else if (dp[i] <= 0.05) { plus = dp[i] + 0.05; minus = 0.0; }
        else { plus = dp[i] + 0.05; minus = dp[i] - 0.05; }
        denom = plus - minus;
        dp[i] = plus;
        grad[i] += yo_offset_interpolate(ds, dp, data) / denom;
        dp[i] = minus;
        grad[i] -= yo_offset_interpolate(ds, dp, data) / denom;
        dp[i] = backup;
        normval += grad[i] * grad[i];
    }
    if (normval != 0.0) {
        normval = sqrt(normval);
        for (i = 0; i < 3; i++) grad[i] /= -normval;
    } else {
        grad[0] = grad[1] = grad[2] = 0.0;
    }
}

/* FIT_eval_transfer_with_light (field_interpolation_tables.pxd:115-143) */
static inline void fit_eval_transfer_with_light(double dt, const double *dvs, const double *grad,
                                                const double *l_dir, const double *l_rgba, double *rgba,
                                                int n_fits, const yo_fit fits[6], const int field_table_ids[6],
                                                int grey_opacity)
{
    int i, fid;
    double ta, dot_prod = 0.0;
    double istorage[6] = {0, 0, 0, 0, 0, 0};
    double trgba[6];
    for (i = 0; i < 3; i++) dot_prod += l_dir[i] * grad[i];
    for (i = 0; i < n_fits; i++) istorage[i] = fit_get(&fits[i], dvs);
    for (i = 0; i < n_fits; i++) {
        fid = fits[i].weight_table_id;
        if (fid != -1) istorage[i] *= istorage[fid];
    }
    for (i = 0; i < 6; i++) trgba[i] = istorage[field_table_ids[i]];
    if (grey_opacity == 1) {
        ta = yo_fmax(1.0 - dt * (trgba[0] + trgba[1] + trgba[2]), 0.0);
        for (i = 0; i < 3; i++) rgba[i] = (1. - ta) * trgba[i] * (1. + dot_prod * l_rgba[i]) + ta * rgba[i];
    } else {
        for (i = 0; i < 3; i++) {
            ta = yo_fmax(1.0 - dt * trgba[i], 0.0);
            rgba[i] = (1. - ta) * trgba[i] * (1. + dot_prod * l_rgba[i]) + ta * rgba[i];
        }
    }
}

/* LightSourceRenderSampler.sample (image_samplers.pyx:551-590): like
 * VolumeRenderSampler.sample without the mask test, with a gradient of
 * field 0 at every sample. */
static void sample_light(const yo_vc *vc, const double v_pos[3], const double v_dir[3],
                         double enter_t, double exit_t, const int index[3], void *data)
{
    yo_acc *im = (yo_acc *)data;
    const yo_sampler *s = im->s;
    int i, j, k;
    int offset = index[0] * (vc->dims[1] + 1) * (vc->dims[2] + 1) + index[1] * (vc->dims[2] + 1) + index[2];
    double dp[3], ds[3], dvs[6] = {0, 0, 0, 0, 0, 0}, grad[3];
    double dt = (exit_t - enter_t) / s->n_samples;
    if (!yo_inside(vc, index)) return;
    for (i = 0; i < 3; i++) {
        dp[i] = (enter_t + 0.5 * dt) * v_dir[i] + v_pos[i];
        dp[i] -= index[i] * vc->dds[i] + vc->left_edge[i];
        dp[i] *= vc->idds[i];
        ds[i] = v_dir[i] * vc->idds[i] * dt;
    }
    for (k = 0; k < s->n_samples; k++) {
        for (j = 0; j < vc->n_fields; j++) dvs[j] = yo_offset_interpolate(vc->dims, dp, vc->data[j] + offset);
        yo_eval_gradient(vc->dims, dp, vc->data[0] + offset, grad);
        fit_eval_transfer_with_light(dt, dvs, grad, s->light_dir, s->light_rgba, im->rgba, s->n_fits, s->fits,
                                     s->field_table_ids, s->grey_opacity);
        for (j = 0; j < 3; j++) dp[j] += ds[j];
    }
}

static void extent_plane_parallel(const yo_sampler *im, const yo_vc *vc, int64_t rv[4])
{
    double temp, cx, cy, extrema[4];
    const double *edges[2];
    int i, j, k;
    edges[0] = vc->left_edge;
    edges[1] = vc->right_edge;
    extrema[0] = extrema[2] = 1e300;
    extrema[1] = extrema[3] = -1e300;
    for (i = 0; i < 2; i++)
        for (j = 0; j < 2; j++)
            for (k = 0; k < 2; k++) {
                temp = edges[i][0] * im->x_vec[0];
                temp += edges[j][1] * im->x_vec[1];
                temp += edges[k][2] * im->x_vec[2];
                if (temp < extrema[0]) extrema[0] = temp;
                if (temp > extrema[1]) extrema[1] = temp;
                temp = edges[i][0] * im->y_vec[0];
                temp += edges[j][1] * im->y_vec[1];
                temp += edges[k][2] * im->y_vec[2];
                if (temp < extrema[2]) extrema[2] = temp;
                if (temp > extrema[3]) extrema[3] = temp;
            }
    cx = cy = 0.0;
    for (i = 0; i < 3; i++) {
        cx += im->center[i] * im->x_vec[i];
        cy += im->center[i] * im->y_vec[i];
    }
    rv[0] = lrint((extrema[0] - cx - im->bounds[0]) / im->pdx);
    rv[1] = rv[0] + lrint((extrema[1] - extrema[0]) / im->pdx);
    rv[2] = lrint((extrema[2] - cy - im->bounds[2]) / im->pdy);
    rv[3] = rv[2] + lrint((extrema[3] - extrema[2]) / im->pdy);
}

static inline double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static void extent_perspective(const yo_sampler *im, const yo_vc *vc, int64_t rv[4])
{
    double cam_pos[3], cam_width[3], north_vector[3], east_vector[3], normal_vector[3];
    double vertex[3], pos1[3], sight_vector[3], sight_center[3];
    float sight_vector_norm, sight_angle_cos, sight_length, dx, dy;
    int i, iv, px, py;
    int min_px = SHRT_MAX, min_py = SHRT_MAX, max_px = -SHRT_MAX, max_py = -SHRT_MAX;
    const double *le = vc->left_edge, *re = vc->right_edge;
    /* corner order of lenses.pyx:83-108 */
    const double cx[8] = {le[0], re[0], re[0], le[0], le[0], re[0], re[0], le[0]};
    const double cy[8] = {le[1], le[1], re[1], re[1], le[1], le[1], re[1], re[1]};
    const double cz[8] = {le[2], le[2], le[2], le[2], re[2], re[2], re[2], re[2]};
    for (i = 0; i < 3; i++) {
        cam_pos[i] = im->camera_data[0 * 3 + i];
        cam_width[i] = im->camera_data[1 * 3 + i];
        east_vector[i] = im->camera_data[2 * 3 + i];
        north_vector[i] = im->camera_data[3 * 3 + i];
        normal_vector[i] = im->camera_data[4 * 3 + i];
    }
    for (iv = 0; iv < 8; iv++) {
        double sn;
        vertex[0] = cx[iv];
        vertex[1] = cy[iv];
        vertex[2] = cz[iv];
        cam_width[1] = cam_width[0] * im->nv[1] / im->nv[0];
        for (i = 0; i < 3; i++) sight_vector[i] = vertex[i] - cam_pos[i];
        for (i = 0; i < 3; i++) sight_center[i] = cam_width[2] * normal_vector[i] + cam_pos[i];
        sn = sqrt(sight_vector[0] * sight_vector[0] + sight_vector[1] * sight_vector[1] +
                  sight_vector[2] * sight_vector[2]);
        sight_vector_norm = (float)sn;
        if (sight_vector_norm != 0)
            for (i = 0; i < 3; i++) sight_vector[i] = sight_vector[i] / (double)sight_vector_norm;
        sight_angle_cos = (float)dot3(sight_vector, normal_vector);
        sight_angle_cos = (float)yo_fclip((double)sight_angle_cos, -1.0, 1.0);
        if (acos((double)sight_angle_cos) < (0.5 * M_PI) && sight_angle_cos != 0.0) {
            sight_length = (float)(cam_width[2] / (double)sight_angle_cos);
        } else {
            sight_length = (float)sqrt(cam_width[0] * cam_width[0] + cam_width[1] * cam_width[1]);
            sight_length = (float)((double)sight_length /
                                   sqrt(1.0 - (double)(sight_angle_cos * sight_angle_cos)));
        }
        for (i = 0; i < 3; i++) pos1[i] = (double)sight_length * sight_vector[i] + cam_pos[i];
        for (i = 0; i < 3; i++) pos1[i] = pos1[i] - sight_center[i];
        dx = (float)dot3(pos1, east_vector);
        dy = (float)dot3(pos1, north_vector);
        px = (int)((im->nv[0] * 0.5) + (((double)im->nv[0] / cam_width[0]) * (double)dx));
        py = (int)((im->nv[1] * 0.5) + (((double)im->nv[1] / cam_width[1]) * (double)dy));
        min_px = min_px < px ? min_px : px;
        max_px = max_px > px ? max_px : px;
        min_py = min_py < py ? min_py : py;
        max_py = max_py > py ? max_py : py;
    }
    rv[0] = min_px > 0 ? min_px : 0;
    rv[1] = max_px < im->nv[0] ? max_px : im->nv[0];
    rv[2] = min_py > 0 ? min_py : 0;
    rv[3] = max_py < im->nv[1] ? max_py : im->nv[1];
}

static void extent_null(const yo_sampler *im, const yo_vc *vc, int64_t rv[4])
{
    (void)vc;
    rv[0] = 0;
    rv[1] = im->nv[0];
    rv[2] = 0;
    rv[3] = im->nv[1];
}

void yo_brick_extent(const yo_sampler *s, const yo_vc *vc, int64_t rv[4])
{
    if (s->extent == 0) extent_plane_parallel(s, vc, rv);
    else if (s->extent == 1) extent_perspective(s, vc, rv);
    else extent_null(s, vc, rv);
}

static inline void vector_info(const yo_sampler *im, int64_t vi, int64_t vj, const double width[3],
                               double v_dir[3], double v_pos[3])
{
    int i;
    if (im->lens == 0) {
        double px, py;
        const double *vp = im->vp_pos;
        px = width[0] * ((double)vi) / ((double)im->nv[0] - 1) - width[0] / 2.0;
        py = width[1] * ((double)vj) / ((double)im->nv[1] - 1) - width[1] / 2.0;
        v_pos[0] = vp[0] * px + vp[3] * py + vp[9];
        v_pos[1] = vp[1] * px + vp[4] * py + vp[10];
        v_pos[2] = vp[2] * px + vp[5] * py + vp[11];
        for (i = 0; i < 3; i++) v_dir[i] = im->vp_dir[i];
    } else {
        int64_t o = (vi * im->nv[1] + vj) * 3;
        for (i = 0; i < 3; i++) {
            v_pos[i] = im->vp_pos[o + i];
            v_dir[i] = im->vp_dir[o + i];
        }
    }
}

static yo_sample_fn pick_sampler(int kind)
{
    switch (kind) {
    case YO_VR: return sample_vr;
    case YO_PROJ: return sample_projection;
    case YO_IPROJ: return sample_interp_proj;
    case YO_LIGHT: return sample_light;
    default: return sample_mip;
    }
}

/* Pixel rectangle a brick covers after yt's +-1 padding and clipping
 * (image_samplers.pyx:159-163). */
void yo_padded_rect(const yo_sampler *s, const yo_vc *vc, int64_t it[4])
{
    yo_brick_extent(s, vc, it);
    it[0] = yo_iclip(it[0] - 1, 0, s->nv[0]);
    it[1] = yo_iclip(it[1] + 1, 0, s->nv[0]);
    it[2] = yo_iclip(it[2] - 1, 0, s->nv[1]);
    it[3] = yo_iclip(it[3] + 1, 0, s->nv[1]);
}

/* cast_through_kdtree for one brick; returns the number of visited cells. */
int64_t yo_cast_through_kdtree(const yo_sampler *s, const yo_vc *vc, int num_threads)
{
    int64_t it[4], nx, ny, size, j;
    int64_t visits = 0;
    double width[3];
    yo_sample_fn fn = pick_sampler(s->kind);
    int i;
    yo_padded_rect(s, vc, it);
    nx = it[1] - it[0];
    ny = it[3] - it[2];
    size = nx * ny;
    if (nx <= 0 || ny <= 0) return 0;
    for (i = 0; i < 3; i++) width[i] = s->width[i];
#ifdef _OPENMP
    if (num_threads <= 0) num_threads = omp_get_max_threads();
#pragma omp parallel for schedule(static, 100) num_threads(num_threads) reduction(+ : visits)
#endif
    for (j = 0; j < size; j++) {
        int64_t vj = j % ny;
        int64_t vi = (j - vj) / ny + it[0];
        double v_pos[3], v_dir[3], max_t;
        yo_acc acc;
        int c;
        double *px;
        vj = vj + it[2];
        vector_info(s, vi, vj, width, v_dir, v_pos);
        px = s->image + (vi * s->nv[1] + vj) * 4;
        for (c = 0; c < 4; c++) acc.rgba[c] = px[c];
        acc.s = s;
        max_t = yo_fclip(s->zbuffer[vi * s->nv[1] + vj], 0.0, 1.0);
        visits += yo_walk_volume(vc, v_pos, v_dir, fn, &acc, NULL, max_t);
        for (c = 0; c < 4; c++) px[c] = acc.rgba[c];
    }
    (void)num_threads;
    return visits;
}

/* Render a brick list in the given order (KDTreeVolumeSource.render's brick
 * loop, render_source.py:594-596). */
int64_t yo_render(const yo_sampler *s, const yo_vc *bricks, const int32_t *order, int64_t n,
                  int num_threads)
{
    int64_t k, visits = 0;
    for (k = 0; k < n; k++) visits += yo_cast_through_kdtree(s, &bricks[order ? order[k] : k], num_threads);
    return visits;
}

/* ---- traversal trace: per-ray FNV-1a over every visited cell -------------- */
typedef struct {
    uint64_t h;
    int64_t n;
    int32_t brick;
} yo_trace_acc;

static inline uint64_t fnv_mix(uint64_t h, uint64_t v)
{
    int b;
    for (b = 0; b < 8; b++) {
        h ^= (v >> (8 * b)) & 0xffu;
        h *= 1099511628211ull;
    }
    return h;
}

uint64_t yo_trace_cell_hash(uint64_t h, int32_t brick, const int index[3], double enter_t, double exit_t)
{
    uint64_t e, x;
    memcpy(&e, &enter_t, 8);
    memcpy(&x, &exit_t, 8);
    h = fnv_mix(h, (uint64_t)(uint32_t)brick);
    h = fnv_mix(h, ((uint64_t)(uint32_t)index[0]) | ((uint64_t)(uint32_t)index[1] << 32));
    h = fnv_mix(h, (uint64_t)(uint32_t)index[2]);
    h = fnv_mix(h, e);
    h = fnv_mix(h, x);
    return h;
}

static void sample_trace(const yo_vc *vc, const double v_pos[3], const double v_dir[3],
                         double enter_t, double exit_t, const int index[3], void *data)
{
    yo_trace_acc *a = (yo_trace_acc *)data;
    (void)vc; (void)v_pos; (void)v_dir;
    a->h = yo_trace_cell_hash(a->h, a->brick, index, enter_t, exit_t);
    a->n += 1;
}

/* For every pixel: hash of all cells visited over the ordered brick list, and
 * the visit count.  hashes/counts are nx*ny, initialised by the caller. */
void yo_trace(const yo_sampler *s, const yo_vc *bricks, const int32_t *order, int64_t n,
              uint64_t *hashes, int64_t *counts, int num_threads)
{
    int64_t k;
    double width[3];
    int i;
    for (i = 0; i < 3; i++) width[i] = s->width[i];
    for (k = 0; k < n; k++) {
        int32_t b = order ? order[k] : (int32_t)k;
        const yo_vc *vc = &bricks[b];
        int64_t it[4], nx, ny, size, j;
        yo_padded_rect(s, vc, it);
        nx = it[1] - it[0];
        ny = it[3] - it[2];
        if (nx <= 0 || ny <= 0) continue;
        size = nx * ny;
#ifdef _OPENMP
        if (num_threads <= 0) num_threads = omp_get_max_threads();
#pragma omp parallel for schedule(static, 100) num_threads(num_threads)
#endif
        for (j = 0; j < size; j++) {
            int64_t vj = j % ny;
            int64_t vi = (j - vj) / ny + it[0];
            double v_pos[3], v_dir[3], max_t;
            yo_trace_acc a;
            int64_t p;
            vj = vj + it[2];
            p = vi * s->nv[1] + vj;
            vector_info(s, vi, vj, width, v_dir, v_pos);
            a.h = hashes[p];
            a.n = counts[p];
            a.brick = b;
            max_t = yo_fclip(s->zbuffer[p], 0.0, 1.0);
            yo_walk_volume(vc, v_pos, v_dir, sample_trace, &a, NULL, max_t);
            hashes[p] = a.h;
            counts[p] = a.n;
        }
    }
}

/* ghost_zone_interpolate (interpolators.pyx:177-226), C-order arrays */
void yo_ghost_zone_interpolate(int rf, const double *in, const int64_t ishape[3], const double input_left[3],
                               double *out, const int64_t oshape[3], const double output_left[3])
{
    int64_t oi, oj, ok;
    int ii, ij, ik, i;
    double xp, xm, yp, ym, zp, zm, temp;
    double ods[3], ids[3], iids[3], opos[3], ropos[3];
#define IN(a, b, c) in[((int64_t)(a) * ishape[1] + (b)) * ishape[2] + (c)]
    for (i = 0; i < 3; i++) {
        temp = input_left[i] + (rf * (ishape[i] - 1));
        ids[i] = (temp - input_left[i]) / (ishape[i] - 1);
        temp = output_left[i] + oshape[i] - 1;
        ods[i] = (temp - output_left[i]) / (oshape[i] - 1);
        iids[i] = 1.0 / ids[i];
    }
    opos[0] = output_left[0];
    for (oi = 0; oi < oshape[0]; oi++) {
        ropos[0] = ((opos[0] - input_left[0]) * iids[0]);
        ii = (int)yo_iclip((int)ropos[0], 0, ishape[0] - 2);
        xp = ropos[0] - ii;
        xm = 1.0 - xp;
        opos[1] = output_left[1];
        for (oj = 0; oj < oshape[1]; oj++) {
            ropos[1] = ((opos[1] - input_left[1]) * iids[1]);
            ij = (int)yo_iclip((int)ropos[1], 0, ishape[1] - 2);
            yp = ropos[1] - ij;
            ym = 1.0 - yp;
            opos[2] = output_left[2];
            for (ok = 0; ok < oshape[2]; ok++) {
                ropos[2] = ((opos[2] - input_left[2]) * iids[2]);
                ik = (int)yo_iclip((int)ropos[2], 0, ishape[2] - 2);
                zp = ropos[2] - ik;
                zm = 1.0 - zp;
                out[(oi * oshape[1] + oj) * oshape[2] + ok] =
                    IN(ii, ij, ik) * (xm * ym * zm) + IN(ii + 1, ij, ik) * (xp * ym * zm) +
                    IN(ii, ij + 1, ik) * (xm * yp * zm) + IN(ii, ij, ik + 1) * (xm * ym * zp) +
                    IN(ii + 1, ij, ik + 1) * (xp * ym * zp) + IN(ii, ij + 1, ik + 1) * (xm * yp * zp) +
                    IN(ii + 1, ij + 1, ik) * (xp * yp * zm) + IN(ii + 1, ij + 1, ik + 1) * (xp * yp * zp);
                opos[2] += ods[2];
            }
            opos[1] += ods[1];
        }
        opos[0] += ods[0];
    }
#undef IN
}

int yo_sizeof_sampler(void) { return (int)sizeof(yo_sampler); }
int yo_sizeof_vc(void) { return (int)sizeof(yo_vc); }

/* ---- per-ray traversal record (for comparison with the reference probe) -- */
typedef struct {
    int64_t n, cap;
    int32_t *cells;
    double *ts;
} yo_rec;

static void sample_record(const yo_vc *vc, const double v_pos[3], const double v_dir[3],
                          double enter_t, double exit_t, const int index[3], void *data)
{
    yo_rec *r = (yo_rec *)data;
    (void)vc; (void)v_pos; (void)v_dir;
    if (r->n < r->cap) {
        r->cells[3 * r->n + 0] = index[0];
        r->cells[3 * r->n + 1] = index[1];
        r->cells[3 * r->n + 2] = index[2];
        r->ts[2 * r->n + 0] = enter_t;
        r->ts[2 * r->n + 1] = exit_t;
    }
    r->n += 1;
}

/* walk_volume for n arbitrary rays through one brick, recording every cell */
void yo_trace_rays(const yo_vc *vc, const double *pos, const double *dir, const double *max_t, int64_t n,
                   int64_t cap, int64_t *counts, int32_t *cells, double *ts)
{
    int64_t i;
    for (i = 0; i < n; i++) {
        yo_rec r;
        r.n = 0;
        r.cap = cap;
        r.cells = cells + 3 * cap * i;
        r.ts = ts + 2 * cap * i;
        yo_walk_volume(vc, pos + 3 * i, dir + 3 * i, sample_record, &r, NULL, max_t[i]);
        counts[i] = r.n;
    }
}

/* ---- octree ray casting --------------------------------------------------
 * Octree<int> of _octree_raytracing.hpp (insert_node :139-175,
 * create_get_node :238-257, cast_ray :199-230, proc_subtree :276-337,
 * first_node / next_node :340-366) and ImageSampler.cast_through_octree
 * (image_samplers.pyx:202-288).  Nodes live in one array; children are
 * indices (-1: none) allocated lazily as the reference allocates them. */
typedef struct {
    int32_t child[8];
    int32_t has_children;
    int32_t terminal;
    int32_t key;
} yo_onode;

typedef struct {
    yo_onode *nodes;
    int64_t n, cap;
    int depth;
    double dle[3], dre[3], size[3];
} yo_octree;

static int32_t yo_onode_new(yo_octree *t)
{
    if (t->n == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 64;
        t->nodes = (yo_onode *)realloc(t->nodes, (size_t)t->cap * sizeof(yo_onode));
    }
    yo_onode *nd = &t->nodes[t->n];
    for (int i = 0; i < 8; i++) nd->child[i] = -1;
    nd->has_children = 0;
    nd->terminal = 0;
    nd->key = 0;
    return (int32_t)t->n++;
}

void *yo_octree_build(int depth, const double *dle, const double *dre, const int32_t *ipos, const int32_t *lvl,
                      const int32_t *key, int64_t n)
{
    yo_octree *t = (yo_octree *)calloc(1, sizeof(yo_octree));
    int64_t c;
    t->depth = depth;
    for (int i = 0; i < 3; i++) {
        t->dle[i] = dle[i];
        t->dre[i] = dre[i];
        t->size[i] = dre[i] - dle[i];
    }
    yo_onode_new(t); /* the root */
    for (c = 0; c < n; c++) {
        uint64_t mask = 1u << (depth - 1);
        int32_t node = 0;
        for (int ibit = depth - 1; ibit >= depth - lvl[c]; --ibit) {
            int iflat = 0;
            for (int d = 0; d < 3; d++) {
                iflat += (ipos[3 * c + d] & mask) != 0;
                iflat <<= 1;
            }
            iflat >>= 1;
            mask >>= 1;
            t->nodes[node].has_children = 1;
            if (t->nodes[node].child[iflat] < 0) {
                int32_t nn = yo_onode_new(t);
                t->nodes[node].child[iflat] = nn;
            }
            node = t->nodes[node].child[iflat];
        }
        t->nodes[node].terminal = 1;
        t->nodes[node].key = key[c];
    }
    return t;
}

void yo_octree_free(void *h)
{
    yo_octree *t = (yo_octree *)h;
    if (!t) return;
    free(t->nodes);
    free(t);
}

static inline double yo_smax(double a, double b) { return (a < b) ? b : a; } /* std::max */
static inline double yo_smin(double a, double b) { return (b < a) ? b : a; } /* std::min */

static int yo_first_node(double tx0, double ty0, double tz0, double txm, double tym, double tzm)
{
    int index = 0;
    if (tx0 >= yo_smax(ty0, tz0)) {
        if (tym < tx0) index |= 2;
        if (tzm < tx0) index |= 1;
    } else if (ty0 >= yo_smax(tx0, tz0)) {
        if (txm < ty0) index |= 4;
        if (tzm < ty0) index |= 1;
    } else {
        if (txm < tz0) index |= 4;
        if (tym < tz0) index |= 2;
    }
    return index;
}

static int yo_next_node(double tx, double ty, double tz, int ix, int iy, int iz)
{
    if (tx < yo_smin(ty, tz)) return ix;
    if (ty < yo_smin(tx, tz)) return iy;
    return iz;
}

typedef void (*yo_ocell_fn)(void *ctx, int32_t key, double t_in, double t_out);

static void yo_proc_subtree(const yo_octree *t, double tx0, double ty0, double tz0, double tx1, double ty1,
                            double tz1, int32_t n, int a, yo_ocell_fn fn, void *ctx)
{
    double txm, tym, tzm;
    int iNode;
    if (tx1 < 0 || ty1 < 0 || tz1 < 0) return;
    if (n < 0) return;
    const yo_onode *nd = &t->nodes[n];
    if (nd->terminal) {
        fn(ctx, nd->key, yo_smax(yo_smax(tx0, ty0), tz0), yo_smin(yo_smin(tx1, ty1), tz1));
        return;
    }
    if (!nd->has_children) return;
    txm = (tx0 + tx1) * 0.5;
    tym = (ty0 + ty1) * 0.5;
    tzm = (tz0 + tz1) * 0.5;
    iNode = yo_first_node(tx0, ty0, tz0, txm, tym, tzm);
    do {
        switch (iNode) {
        case 0:
            yo_proc_subtree(t, tx0, ty0, tz0, txm, tym, tzm, nd->child[a], a, fn, ctx);
            iNode = yo_next_node(txm, tym, tzm, 4, 2, 1);
            break;
        case 1:
            yo_proc_subtree(t, tx0, ty0, tzm, txm, tym, tz1, nd->child[1 ^ a], a, fn, ctx);
            iNode = yo_next_node(txm, tym, tz1, 5, 3, 8);
            break;
        case 2:
            yo_proc_subtree(t, tx0, tym, tz0, txm, ty1, tzm, nd->child[2 ^ a], a, fn, ctx);
            iNode = yo_next_node(txm, ty1, tzm, 6, 8, 3);
            break;
        case 3:
            yo_proc_subtree(t, tx0, tym, tzm, txm, ty1, tz1, nd->child[3 ^ a], a, fn, ctx);
            iNode = yo_next_node(txm, ty1, tz1, 7, 8, 8);
            break;
        case 4:
            yo_proc_subtree(t, txm, ty0, tz0, tx1, tym, tzm, nd->child[4 ^ a], a, fn, ctx);
            iNode = yo_next_node(tx1, tym, tzm, 8, 6, 5);
            break;
        case 5:
            yo_proc_subtree(t, txm, ty0, tzm, tx1, tym, tz1, nd->child[5 ^ a], a, fn, ctx);
            iNode = yo_next_node(tx1, tym, tz1, 8, 7, 8);
            break;
        case 6:
            yo_proc_subtree(t, txm, tym, tz0, tx1, ty1, tzm, nd->child[6 ^ a], a, fn, ctx);
            iNode = yo_next_node(tx1, ty1, tzm, 8, 8, 7);
            break;
        case 7:
            yo_proc_subtree(t, txm, tym, tzm, tx1, ty1, tz1, nd->child[7 ^ a], a, fn, ctx);
            iNode = 8;
            break;
        }
    } while (iNode < 8);
}

/* Octree::cast_ray (Ray normalises the direction, :49-64) */
static void yo_octree_cast_ray(const yo_octree *t, const double *o_in, const double *d_in, yo_ocell_fn fn,
                               void *ctx)
{
    double o[3], d[3], dd = 0, t0[3], t1[3], tmax0, tmin1;
    int a = 0, bmask = 4, i;
    for (i = 0; i < 3; i++) o[i] = o_in[i];
    for (i = 0; i < 3; i++) dd += d_in[i] * d_in[i];
    dd = sqrt(dd);
    for (i = 0; i < 3; i++) d[i] = d_in[i] / dd;
    for (i = 0; i < 3; i++) {
        if (d[i] < 0.0) {
            o[i] = t->size[i] - o[i];
            d[i] = -d[i];
            a |= bmask;
        }
        bmask >>= 1;
    }
    for (i = 0; i < 3; i++) {
        t0[i] = (t->dle[i] - o[i]) / d[i];
        t1[i] = (t->dre[i] - o[i]) / d[i];
    }
    tmax0 = t0[0];  /* std::max_element: the first largest */
    for (i = 1; i < 3; i++) if (tmax0 < t0[i]) tmax0 = t0[i];
    tmin1 = t1[0];  /* std::min_element: the first smallest */
    for (i = 1; i < 3; i++) if (t1[i] < tmin1) tmin1 = t1[i];
    if (tmax0 < tmin1) yo_proc_subtree(t, t0[0], t0[1], t0[2], t1[0], t1[1], t1[2], 0, a, fn, ctx);
}

typedef struct {
    const yo_sampler *s;
    const double *cells;  /* 14 per cell: 8 vertex values, left edge, right edge */
    const double *v_pos, *v_dir;
    double len;
    yo_acc *acc;
    yo_sample_fn fn;
    int64_t visits;
    /* trace mode */
    uint64_t h;
    int64_t count;
} yo_octx;

static void yo_octree_cell(void *vctx, int32_t key, double t_in, double t_out)
{
    yo_octx *c = (yo_octx *)vctx;
    yo_vc vc;
    int k;
    uint8_t mask[8] = {1, 1, 1, 1, 1, 1, 1, 1};
    int index[3] = {0, 0, 0};
    const double *cd = c->cells + 14 * (int64_t)key;
    vc.n_fields = 1;
    vc.data[0] = cd;
    vc.mask = mask;
    for (k = 0; k < 3; k++) {
        vc.dims[k] = 1;
        vc.left_edge[k] = cd[8 + k];
        vc.right_edge[k] = cd[11 + k];
        vc.dds[k] = (vc.right_edge[k] - vc.left_edge[k]);
        vc.idds[k] = 1 / vc.dds[k];
    }
    c->visits++;
    if (c->fn) {
        c->fn(&vc, c->v_pos, c->v_dir, t_in / c->len, t_out / c->len, index, c->acc);
    } else {
        double e = t_in / c->len, x = t_out / c->len;
        uint64_t eb, xb;
        memcpy(&eb, &e, 8);
        memcpy(&xb, &x, 8);
        /* a NaN enters the hash as one pattern: its sign and payload differ
         * between x86, Arm and the GPU */
        if (e != e) eb = 0x7ff8000000000000ull;
        if (x != x) xb = 0x7ff8000000000000ull;
        c->h = fnv_mix(c->h, (uint64_t)(uint32_t)key);
        c->h = fnv_mix(c->h, eb);
        c->h = fnv_mix(c->h, xb);
        c->count++;
    }
}

/* cast_through_octree over the per-pixel rays of s (lens 1); returns the
 * number of cells sampled.  With hashes/counts set, records per pixel an
 * FNV-1a hash over (cell key, enter bits, exit bits) instead of sampling. */
int64_t yo_cast_through_octree(const yo_sampler *s, const double *cells, const void *octree, int num_threads,
                               uint64_t *hashes, int64_t *counts)
{
    const yo_octree *t = (const yo_octree *)octree;
    int64_t j, size = (int64_t)s->nv[0] * s->nv[1], visits = 0;
    yo_sample_fn fn = hashes ? NULL : pick_sampler(s->kind);
    if (s->lens != 1) return -1;
#ifdef _OPENMP
    if (num_threads <= 0) num_threads = omp_get_max_threads();
#pragma omp parallel for schedule(static, 100) num_threads(num_threads) reduction(+ : visits)
#endif
    for (j = 0; j < size; j++) {
        int64_t vj = j % s->nv[1];
        int64_t vi = (j - vj) / s->nv[1];
        const double *vp = s->vp_pos + (vi * s->nv[1] + vj) * 3;
        const double *vd = s->vp_dir + (vi * s->nv[1] + vj) * 3;
        yo_acc acc;
        yo_octx c;
        double *px = s->image + (vi * s->nv[1] + vj) * 4;
        int k;
        c.s = s;
        c.cells = cells;
        c.v_pos = vp;
        c.v_dir = vd;
        c.len = sqrt(pow(vd[0], 2.0) + pow(vd[1], 2.0) + pow(vd[2], 2.0));
        c.acc = &acc;
        c.fn = fn;
        c.visits = 0;
        c.h = hashes ? hashes[j] : 0;
        c.count = 0;
        for (k = 0; k < 4; k++) acc.rgba[k] = px[k];
        acc.s = s;
        yo_octree_cast_ray(t, vp, vd, yo_octree_cell, &c);
        if (c.visits > 0 && !hashes)
            for (k = 0; k < 4; k++) px[k] = acc.rgba[k];
        if (hashes) {
            hashes[j] = c.h;
            counts[j] += c.count;
        }
        visits += c.visits;
    }
    (void)num_threads;
    return visits;
}

/* ---- octree off-axis projection: cell splatting ---------------------------
 * add_cells_to_image_offaxis (image_utilities.pyx:167-289) with its stamp
 * precomputation (direct_integrate_cube :321-407, check_in_parallelogram
 * :296-318) and per-cell splat (_add_cell_to_image_offaxis :46-165),
 * restated sequentially: one accumulation buffer instead of one per
 * thread (the reference's thread buffers are summed in an unspecified
 * order), and the stamp normalised by a left-to-right sum (numpy's pairwise
 * sum in the reference; the two agree to a few ulps). */

static double oa_fmax(double a, double b) { return a > b ? a : b; } /* fp_utils.pxd */
static double oa_fmin(double a, double b) { return a < b ? a : b; }
static double oa_fclip(double f, double a, double b) { return oa_fmin(oa_fmax(f, a), b); }

static int oa_in_parallelogram(const double PA[2], const double PQ[2], const double PR[2], int sPQ, int sPR,
                               double out[2])
{
    double det = PQ[0] * PR[1] - PQ[1] * PR[0];
    if (det == 0) return 0;
    out[0] = -(PA[0] * PQ[1] - PA[1] * PQ[0]) / det;
    out[1] = (PA[0] * PR[1] - PA[1] * PR[0]) / det;
    return 0 <= sPQ * out[0] && sPQ * out[0] <= 1 && 0 <= sPR * out[1] && sPR * out[1] <= 1;
}

/* depth of the unit cube spanned by u, v, w from O at the centres of an
 * nx x ny grid, into buf/mask rows of length stride; -1 on a single hit */
static int oa_integrate_cube(const double O[3], const double u[3], const double v[3], const double w[3],
                             double *buf, uint8_t *mask, int nx, int ny, int stride)
{
    double Ob[3], F[2], B[2], nm[2];
    int i, j, k;
    for (k = 0; k < 3; k++) Ob[k] = O[k] + u[k] + v[k] + w[k];
    for (i = 0; i < nx; i++) {
        double X0 = (i + 0.5) * (1. / nx);
        F[0] = X0 - O[0];
        B[0] = X0 - Ob[0];
        for (j = 0; j < ny; j++) {
            double X1 = (j + 0.5) * (1. / ny), zmin = INFINITY, zmax = -INFINITY, z;
            int nhit = 0;
            F[1] = X1 - O[1];
            B[1] = X1 - Ob[1];
#define OA_FACE(PA, P, R, s, Z0, c0, c1)                                                                   \
    if (oa_in_parallelogram(PA, P, R, s, s, nm)) {                                                         \
        z = Z0 + nm[0] * c0 + nm[1] * c1;                                                                  \
        zmin = oa_fmin(z, zmin);                                                                           \
        zmax = oa_fmax(z, zmax);                                                                           \
        nhit++;                                                                                            \
    }
            OA_FACE(F, v, u, 1, O[2], u[2], v[2])
            OA_FACE(F, w, v, 1, O[2], v[2], w[2])
            OA_FACE(F, w, u, 1, O[2], u[2], w[2])
            OA_FACE(B, v, u, -1, Ob[2], u[2], v[2])
            OA_FACE(B, w, v, -1, Ob[2], v[2], w[2])
            OA_FACE(B, w, u, -1, Ob[2], u[2], w[2])
#undef OA_FACE
            if (nhit == 1) return -1;
            if (nhit > 1) {
                buf[i * stride + j] += zmax - zmin;
                mask[i * stride + j] = 1;
            }
        }
    }
    return 0;
}

/* the stamp's extent (image_utilities.pyx:220-225) */
void yo_offaxis_extent(double dx_max, int nx, int ny, int npix_min, int32_t out[3])
{
    int nsx = (int)ceil(2 * dx_max * sqrt(3) * nx), nsy = (int)ceil(2 * dx_max * sqrt(3) * ny);
    if (nsx < npix_min) nsx = npix_min;
    if (nsy < npix_min) nsy = npix_min;
    out[0] = nsx;
    out[1] = nsy;
    out[2] = (int)ceil(log2((double)(nsx > nsy ? nsx : nsy)));
}

/* the stamps (image_utilities.pyx:204-246) into stamp / mask
 * (max_depth, nsx, nsy), zeroed by the caller; rot is the 3x3 rotation,
 * row-major.  Returns -1 where the reference raises. */
int yo_offaxis_stamp(const double *rot, int nsx, int nsy, int max_depth, double *stamp, uint8_t *mask)
{
    double w0 = 1 / sqrt(3.), e[3][3] = {{0}}, abc[3][3], o[3];
    int i, k, d;
    for (i = 0; i < 3; i++) e[i][i] = 1. * w0;
    for (i = 0; i < 3; i++)
        for (k = 0; k < 3; k++)
            abc[i][k] = rot[3 * k] * e[i][0] + rot[3 * k + 1] * e[i][1] + rot[3 * k + 2] * e[i][2];
    for (k = 0; k < 3; k++) o[k] = 0.5 - (abc[0][k] + abc[1][k] + abc[2][k]) / 2;
    for (d = 0; d < max_depth; d++) {
        double *s = stamp + (int64_t)d * nsx * nsy, sum = 0;
        int64_t m;
        if (d == 0) {
            s[0] = 1;
            continue;
        }
        if (oa_integrate_cube(o, abc[0], abc[1], abc[2], s, mask + (int64_t)d * nsx * nsy,
                              (1 << d) < nsx ? (1 << d) : nsx, (1 << d) < nsy ? (1 << d) : nsy, nsy) < 0)
            return -1;
        for (m = 0; m < (int64_t)nsx * nsy; m++) sum += s[m];
        for (m = 0; m < (int64_t)nsx * nsy; m++) s[m] /= sum;
    }
    return 0;
}

static void oa_add(double *b, double *bw, int64_t idx, int64_t npix, double vq, double vw)
{
    if (idx >= 0 && idx < npix) {
        b[idx] += vq;
        bw[idx] += vw;
    }
}

/* _add_cell_to_image_offaxis (image_utilities.pyx:46-165) for one cell into
 * the linear buffers b / bw (pixel (i, j) at i * nx + j) */
static void oa_cell(double dx, double w, double q, double cmw, double x, double y, int nx, int ny, int nsx,
                    int nsy, double *b, double *bw, int max_depth, const double *stamp, const uint8_t *mask)
{
    double half = cmw / 2, dx3 = dx * dx * dx * nx * ny, lx = x - half, rx = x + half, ly = y - half,
           ry = y + half, dx_loc, dy_loc;
    int64_t npix = (int64_t)nx * ny;
    int jmin = (int)floor(lx * nx), jmax = (int)ceil(rx * nx), kmin = (int)floor(ly * ny),
        kmax = (int)ceil(ry * ny), depth, j, k;
    if (jmin < 0) jmin = 0;
    if (jmax < nx - 1) jmax = nx - 1;
    if (kmin > 0) kmin = 0;
    if (kmax < ny - 1) kmax = ny - 1;
    if (jmax == jmin + 1 && kmax == kmin + 1) {
        oa_add(b, bw, (int64_t)jmin * nx + kmin, npix, q * dx3, w * dx3);
        return;
    }
    depth = (int)ceil(log2(4 * sqrt(3) * dx * oa_fmax(nx, ny)));
    if (depth < 1) depth = 1;
    if (depth > max_depth - 1) depth = max_depth - 1;
    jmax = nsx < (1 << depth) ? nsx : (1 << depth);
    kmax = nsy < (1 << depth) ? nsy : (1 << depth);
    dx_loc = cmw / jmax;
    dy_loc = cmw / kmax;
    for (j = 0; j < jmax; j++) {
        double xx1 = ((j - jmax / 2.) * dx_loc + x) * nx, xx2 = ((j + 1 - jmax / 2.) * dx_loc + x) * nx, dvx;
        int jj1 = (int)xx1, jj2 = (int)xx2;
        if (jj2 < 0 || jj1 >= nx) continue;
        dvx = oa_fclip((jj2 - xx1) / (xx2 - xx1), 0., 1.);
        for (k = 0; k < kmax; k++) {
            int64_t si = ((int64_t)depth * nsx + j) * nsy + k;
            double yy1, yy2, tmp, sw, sq, dvy;
            int kk1, kk2;
            if (mask[si] == 0) continue;
            yy1 = ((k - kmax / 2.) * dy_loc + y) * ny;
            yy2 = ((k + 1 - kmax / 2.) * dy_loc + y) * ny;
            kk1 = (int)yy1;
            kk2 = (int)yy2;
            if (kk2 < 0 || kk1 >= ny) continue;
            tmp = stamp[si] * dx3;
            sw = tmp * w;
            sq = tmp * q;
            dvy = oa_fclip((kk2 - yy1) / (yy2 - yy1), 0., 1.);
            if (jj1 >= 0 && kk1 >= 0) {
                tmp = dvx * dvy;
                oa_add(b, bw, (int64_t)jj1 * nx + kk1, npix, sq * tmp, sw * tmp);
            }
            if (jj1 >= 0 && kk2 < ny) {
                tmp = dvx * (1 - dvy);
                oa_add(b, bw, (int64_t)jj1 * nx + kk2, npix, sq * tmp, sw * tmp);
            }
            if (jj2 < nx && kk1 >= 0) {
                tmp = (1 - dvx) * dvy;
                oa_add(b, bw, (int64_t)jj2 * nx + kk1, npix, sq * tmp, sw * tmp);
            }
            if (jj2 < nx && kk2 < ny) {
                tmp = (1 - dvx) * (1 - dvy);
                oa_add(b, bw, (int64_t)jj2 * nx + kk2, npix, sq * tmp, sw * tmp);
            }
        }
    }
}

/* The cell loop of add_cells_to_image_offaxis (image_utilities.pyx:249-289):
 * every cell into a zeroed linear buffer, then buffer[j, k] += linear[j *
 * nx + k] for the (nx, ny) C-order outputs.  Returns -1 for nx > ny (the
 * reference then writes outside its buffer) or on allocation failure. */
int yo_add_cells_offaxis(const double *xp, const double *dxp, const double *qty, const double *weight, int64_t n,
                         const double *rot, const double *stamp, const uint8_t *mask, int nsx, int nsy,
                         int max_depth, int nx, int ny, double *buffer, double *buffer_weight)
{
    int64_t i, npix = (int64_t)nx * ny;
    double *lb, *lbw, sq3 = sqrt(3.);
    int j, k;
    if (nx > ny) return -1;
    lb = (double *)calloc((size_t)npix, sizeof(double));
    lbw = (double *)calloc((size_t)npix, sizeof(double));
    if (!lb || !lbw) {
        free(lb);
        free(lbw);
        return -1;
    }
    for (i = 0; i < n; i++) {
        double dx = dxp[i], cmw = dx * sq3;
        double x = (rot[0] * xp[3 * i] + rot[1] * xp[3 * i + 1] + rot[2] * xp[3 * i + 2]) + 0.5;
        double y = (rot[3] * xp[3 * i] + rot[4] * xp[3 * i + 1] + rot[5] * xp[3 * i + 2]) + 0.5;
        oa_cell(dx, weight[i], qty[i], cmw, x, y, nx, ny, nsx, nsy, lb, lbw, max_depth, stamp, mask);
    }
    for (j = 0; j < nx; j++)
        for (k = 0; k < ny; k++) {
            buffer[(int64_t)j * ny + k] += lb[(int64_t)j * nx + k];
            buffer_weight[(int64_t)j * ny + k] += lbw[(int64_t)j * nx + k];
        }
    free(lb);
    free(lbw);
    return 0;
}
