// ytgb_render.cu -- the per-pixel-ray sampler kernels of libytgb (sm_103a).
//
// One CUDA thread owns one pixel ray for the whole launch and walks every
// brick of the view in the kd viewpoint order, so the per-brick Python loop,
// OpenMP region and image read/write of yt's cast_through_kdtree
// (image_samplers.pyx:146-197) disappear.  Each block bins the ordered brick
// list against its 8x16 pixel tile (the bricks' pixel rectangles) in shared
// memory, so a ray only looks at bricks whose rectangle can contain it.
//
// Precision split.  The cell walk of walk_volume (grid_traversal.pyx:26-140)
// is reproduced bit for bit: every float64 value the walk compares or hands
// to its sampler (intersect_t, tmax, tdelta, enter_t, exit_t, the cell index)
// is computed from the same operands in the same order as the reference, as
// _rn intrinsics (never contracted).  On GB300 the float64 pipe is far slower
// than float32, so everything else is kept off it:
//   * comparisons of walk values use order-preserving int64 keys;
//   * per cell only `tmax += tdelta` and `exit_t - enter_t` run in float64;
//   * the sample position is tracked in float32, in cell-local coordinates
//     reset exactly on the axis the walk steps along;
//   * bricks a ray clearly misses, faces it clearly does not enter through,
//     and start points clearly outside a brick are rejected by float32 tests
//     whose margins exceed their float32 error by orders of magnitude, before
//     the exact float64 tests;
//   * tdelta (a function of the ray and the brick's dds only) is reused
//     across bricks of equal dds.
// Sampling (trilinear, transfer function) runs in float32 on float32 brick
// data.  The image accumulates as a float32 value plus a float32 error term
// with error-free transformations (TwoSum, Knuth; TwoProduct via FMA), so
// rounding stays at the level of one float32 rounding per sample instead of
// growing with the ray length.
//
// The per-ray brick walk lives in ytgb_ray.cuh (host/device code, so the
// test harness can run it on the CPU); this file holds the kernels.
//
// Out-of-brick cells.  walk_volume can hand its sampler an index outside the
// brick: on an axis with v_dir == 0 whose start point was snapped onto a face
// from just outside (grid_traversal.pyx:67-78) the index is -1, and the
// jump-start test (:113-117) only rejects -1 for negative steps.  yt then
// reads outside the brick's arrays.  Here such a cell contributes nothing and
// is counted in counters[3]; the trace still records it.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "ytgb.h"
#include "ytgb_internal.h"
#include "ytgb_ray.cuh"

namespace {

using namespace ytgb;

constexpr int TILE_X = 8;    // image rows (vi) per block
constexpr int TILE_Y = 16;   // image columns (vj) per block
constexpr int BLOCK = TILE_X * TILE_Y;
constexpr int NWARP = BLOCK / 32;

// CTF = 1: ColorTransferFunction layout -- one bin lookup serves all four
// tables, packed per bin in shared memory as y[4], dy[4] and the d0 pair.
template <int MODE, int CTF>
__global__ void __launch_bounds__(BLOCK) render_kernel(const ytgb_render_args a, unsigned long long *hashes,
                                                       long long *counts) {
    extern __shared__ float4 s_tab[];
    __shared__ unsigned long long s_cnt[4];
    __shared__ int s_sel[BLOCK];
    __shared__ int s_wsum[NWARP];
    const ytgb_view &v = a.view;
    const int tid = threadIdx.x;
    if (tid < 4) s_cnt[tid] = 0;
    if (MODE == MODE_VR) {
        const float4 *g = reinterpret_cast<const float4 *>(a.tf_tables);
        if (CTF) {
            const int nb = a.tf.nbins_max;
            for (int b = tid; b < nb; b += BLOCK) {
                float4 t0 = __ldg(g + 0 * nb + b), t1 = __ldg(g + 1 * nb + b);
                float4 t2 = __ldg(g + 2 * nb + b), t3 = __ldg(g + 3 * nb + b);
                s_tab[3 * b + 0] = make_float4(t0.x, t1.x, t2.x, t3.x);
                s_tab[3 * b + 1] = make_float4(t0.y, t1.y, t2.y, t3.y);
                s_tab[3 * b + 2] = make_float4(t3.z, t3.w, 0.f, 0.f);
            }
        } else {
            const int n = a.tf.n_fits * a.tf.nbins_max;
            for (int k = tid; k < n; k += BLOCK) s_tab[k] = __ldg(g + k);
        }
    }
    __syncthreads();

    const int vj = blockIdx.x * TILE_Y + (tid % TILE_Y);
    const int vi = blockIdx.y * TILE_X + (tid / TILE_Y);
    const bool active = vi < v.nx && vj < v.ny;
    const int tx0 = blockIdx.y * TILE_X, tx1 = tx0 + TILE_X;
    const int ty0 = blockIdx.x * TILE_Y, ty1 = ty0 + TILE_Y;
    const size_t p = active ? (size_t)vi * v.ny + vj : 0;

    Ray r;
    if (active) make_ray(v, vi, vj, r);
    double *img = a.image + p * 4;
    RayState st;
    ray_state_init(st, (active && MODE != MODE_TRACE) ? img : nullptr, (active && a.zbuffer) ? a.zbuffer[p] : 1.0,
                   a.zbuffer != nullptr, a.flags);
    if (MODE == MODE_TRACE && active) {
        st.th = hashes[p];
        st.tcount = counts[p];
    }
    const int4 *rects = reinterpret_cast<const int4 *>(a.rects);

    for (int base = 0; base < a.n_order; base += BLOCK) {
        // ---- bin the next BLOCK bricks against this block's pixel tile -------
        const int k = base + tid;
        bool hit = false;
        if (k < a.n_order) {
            const int4 rc = __ldg(rects + k);
            hit = rc.x < tx1 && rc.y > tx0 && rc.z < ty1 && rc.w > ty0;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        const int lane = tid & 31, wid = tid >> 5;
        if (lane == 0) s_wsum[wid] = __popc(bal);
        __syncthreads();
        int off = 0, nsel = 0;
#pragma unroll
        for (int q = 0; q < NWARP; q++) {
            off += q < wid ? s_wsum[q] : 0;
            nsel += s_wsum[q];
        }
        if (hit) s_sel[off + __popc(bal & ((1u << lane) - 1u))] = k;
        __syncthreads();

        for (int j = 0; active && j < nsel; j++) {
            const int kk = s_sel[j];
            const int4 rc = __ldg(rects + kk);
            if (vi < rc.x || vi >= rc.y || vj < rc.z || vj >= rc.w) continue;
            walk_brick<MODE, CTF>(a, s_tab, r, __ldg(a.order + kk), st);
        }
        __syncthreads();  // s_sel is rewritten by the next chunk
    }

    if (active) {
        if (MODE == MODE_TRACE) {
            hashes[p] = st.th;
            counts[p] = st.tcount;
        } else {
#pragma unroll
            for (int c = 0; c < 4; c++)
                if (st.touched & (1u << c)) img[c] = (double)st.xh[c] + (double)st.xl[c];
        }
    }
    if (a.counters) {
        if (st.visits) atomicAdd(&s_cnt[0], st.visits);
        if (st.walks) atomicAdd(&s_cnt[1], st.walks);
        if (st.guarded) atomicAdd(&s_cnt[3], st.guarded);
        if (active) atomicAdd(&s_cnt[2], 1ull);
        __syncthreads();
        if (tid < 4 && s_cnt[tid]) atomicAdd(a.counters + tid, s_cnt[tid]);
    }
}

int check_args(const ytgb_render_args *a, bool trace) {
    if (!a) {
        ytgb_set_error("ytgb_render: null args");
        return YTGB_ERR_INVALID;
    }
    const ytgb_view &v = a->view;
    if (v.nx <= 0 || v.ny <= 0) {
        ytgb_set_error("ytgb_render: empty image");
        return YTGB_ERR_INVALID;
    }
    if (a->kind < 0 || a->kind > 3) {
        ytgb_set_error("ytgb_render: unknown sampler kind");
        return YTGB_ERR_INVALID;
    }
    if (a->n_order < 0 || (a->n_order > 0 && (!a->order || !a->rects || !a->bricks || !a->data))) {
        ytgb_set_error("ytgb_render: missing brick arrays");
        return YTGB_ERR_INVALID;
    }
    if (!trace && !a->image) {
        ytgb_set_error("ytgb_render: missing image");
        return YTGB_ERR_INVALID;
    }
    if (v.lens == YTGB_LENS_PER_PIXEL && (!v.px_pos || !v.px_dir)) {
        ytgb_set_error("ytgb_render: per-pixel lens needs px_pos / px_dir");
        return YTGB_ERR_INVALID;
    }
    if (v.lens != YTGB_LENS_PER_PIXEL && v.lens != YTGB_LENS_PLANE_PARALLEL) {
        ytgb_set_error("ytgb_render: unknown lens");
        return YTGB_ERR_INVALID;
    }
    if (a->n_samples < 1) {
        ytgb_set_error("ytgb_render: n_samples must be >= 1");
        return YTGB_ERR_INVALID;
    }
    if (!trace && a->kind == YTGB_VOLUME_RENDER && !a->tf_tables) {
        ytgb_set_error("ytgb_render: volume rendering needs a transfer function");
        return YTGB_ERR_INVALID;
    }
    return YTGB_OK;
}

template <int MODE, int CTF>
int launch(const ytgb_render_args *a, size_t smem, cudaStream_t s, unsigned long long *h, long long *c) {
    dim3 grid((a->view.ny + TILE_Y - 1) / TILE_Y, (a->view.nx + TILE_X - 1) / TILE_X);
    if (grid.y > 65535) {
        ytgb_set_error("ytgb_render: image too tall");
        return YTGB_ERR_INVALID;
    }
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(render_kernel<MODE, CTF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            ytgb_set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return YTGB_ERR_CUDA;
        }
    }
    render_kernel<MODE, CTF><<<grid, BLOCK, smem, s>>>(*a, h, c);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("render launch: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return YTGB_OK;
}

}  // namespace

extern "C" int ytgb_render(const ytgb_render_args *a, void *stream) {
    int st = check_args(a, false);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (a->kind == YTGB_VOLUME_RENDER) {
        const ytgb_tf &t = a->tf;
        if (t.n_fits < 0 || t.n_fits > 6 || t.nbins_max < 2 || t.nbins_max > YTGB_TF_MAX_BINS) {
            ytgb_set_error("ytgb_render: inconsistent transfer function header");
            return YTGB_ERR_INVALID;
        }
        for (int q = 0; q < t.n_fits; q++) {
            if (t.nbins[q] < 2 || t.nbins[q] > t.nbins_max || t.field_id[q] < 0 || t.field_id[q] > 5 ||
                t.weight_field_id[q] < -1 || t.weight_field_id[q] > 5 || t.weight_table_id[q] < -1 ||
                t.weight_table_id[q] >= t.n_fits) {
                ytgb_set_error("ytgb_render: transfer function table ids out of range");
                return YTGB_ERR_INVALID;
            }
        }
        for (int c = 0; c < 6; c++) {
            if (t.field_table_ids[c] < 0 || t.field_table_ids[c] > 5) {
                ytgb_set_error("ytgb_render: field_table_ids out of range");
                return YTGB_ERR_INVALID;
            }
        }
        if (t.ctf_fast && (t.n_fits != 4 || t.nbins[0] != t.nbins_max)) {
            ytgb_set_error("ytgb_render: ctf_fast set on tables that are not a ColorTransferFunction");
            return YTGB_ERR_INVALID;
        }
        const size_t smem = t.ctf_fast ? (size_t)3 * t.nbins_max * sizeof(float4)
                                       : (size_t)t.n_fits * t.nbins_max * sizeof(float4);
        if (smem > 200 * 1024) {
            ytgb_set_error("ytgb_render: transfer-function tables exceed 200 KB of shared memory");
            return YTGB_ERR_INVALID;
        }
        return t.ctf_fast ? launch<MODE_VR, 1>(a, smem, s, nullptr, nullptr)
                          : launch<MODE_VR, 0>(a, smem, s, nullptr, nullptr);
    }
    switch (a->kind) {
    case YTGB_PROJECTION: return launch<MODE_PROJ, 0>(a, 0, s, nullptr, nullptr);
    case YTGB_INTERPOLATED_PROJECTION: return launch<MODE_IPROJ, 0>(a, 0, s, nullptr, nullptr);
    default: return launch<MODE_MIP, 0>(a, 0, s, nullptr, nullptr);
    }
}

extern "C" int ytgb_trace(const ytgb_render_args *a, unsigned long long *hashes, long long *counts, void *stream) {
    int st = check_args(a, true);
    if (st) return st;
    if (!hashes || !counts) {
        ytgb_set_error("ytgb_trace: null hash / count arrays");
        return YTGB_ERR_INVALID;
    }
    return launch<MODE_TRACE, 0>(a, 0, (cudaStream_t)stream, hashes, counts);
}

extern "C" int ytgb_check_error(const int32_t *d_error, void *stream) {
    if (!d_error) return YTGB_OK;
    int32_t h = 0;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(&h, d_error, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("ytgb_check_error: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    if (h != 0) {
        char buf[96];
        snprintf(buf, sizeof(buf), "device guard tripped (code %d)", (int)h);
        ytgb_set_error(buf);
        e = cudaMemsetAsync(const_cast<int32_t *>(d_error), 0, sizeof(int32_t), s);
        return YTGB_ERR_DEVICE;
    }
    return YTGB_OK;
}
