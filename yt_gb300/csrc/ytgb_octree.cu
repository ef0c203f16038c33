// ytgb_octree.cu -- the octree sampler path (cast_through_octree).
//
// One thread per pixel ray: the octree traversal of ytgb_octree.cuh, and for
// each terminal cell the same sampler code the kd path runs
// (ytgb_ray.cuh:sample_cell) on a 1x1x1 brick with the cell's edges, as
// ImageSampler.cast_through_octree (image_samplers.pyx:202-288) does.  The
// octree path has no zbuffer (the reference ignores it there) and no masks.
#include <cuda_runtime.h>
#include <cstdint>
#include <string>

#include "ytgb.h"
#include "ytgb_internal.h"
#include "ytgb_octree.cuh"

namespace {

using namespace ytgb;

constexpr int OBLOCK = 128;
// A block renders a 16 x 8 pixel tile, each warp an 8 x 4 sub-tile: rays
// that traverse the octree together stay close on the image, so a warp's
// lanes follow more of the same path than along a 32-pixel row.
constexpr int OTILE_X = 16, OTILE_Y = 8;

static_assert(sizeof(ytgb_onode) == sizeof(ONode), "ytgb_onode layout");

template <int MODE, int CTF>
__global__ void __launch_bounds__(OBLOCK) octree_kernel(const ytgb_render_args a, const ytgb_octree_args oa,
                                                         unsigned long long *hashes, long long *counts) {
    extern __shared__ float4 s_tab[];
    __shared__ unsigned long long s_cnt[4];
    const int tid = threadIdx.x;
    if (tid < 4) s_cnt[tid] = 0;
    if (MODE == MODE_VR || MODE == MODE_LIGHT) {
        const float4 *g = reinterpret_cast<const float4 *>(a.tf_tables);
        const int nb = a.tf.nbins_max;
        if (CTF) {
            for (int b = tid; b < nb; b += OBLOCK) {
                float4 t0 = __ldg(g + 0 * nb + b), t1 = __ldg(g + 1 * nb + b);
                float4 t2 = __ldg(g + 2 * nb + b), t3 = __ldg(g + 3 * nb + b);
                s_tab[3 * b + 0] = make_float4(t0.x, t1.x, t2.x, t3.x);
                s_tab[3 * b + 1] = make_float4(t0.y, t1.y, t2.y, t3.y);
                s_tab[3 * b + 2] = make_float4(t3.z, t3.w, 0.f, 0.f);
            }
        } else {
            const int n = a.tf.n_fits * nb;
            for (int k = tid; k < n; k += OBLOCK) s_tab[k] = __ldg(g + k);
        }
    }
    __syncthreads();
    const ytgb_view &v = a.view;
    const int tiles_y = (v.ny + OTILE_Y - 1) / OTILE_Y;
    const int warp = tid >> 5, lane = tid & 31;
    const int vi = (int)(blockIdx.x / tiles_y) * OTILE_X + (warp & 1) * 8 + (lane & 7);
    const int vj = (int)(blockIdx.x % tiles_y) * OTILE_Y + (warp >> 1) * 4 + (lane >> 3);
    const bool active = vi < v.nx && vj < v.ny;
    const long long p = (long long)vi * v.ny + vj;
    RayState st;
    double *img = active ? a.image + p * 4 : nullptr;
    ray_state_init(st, MODE != MODE_TRACE ? img : nullptr, 1.0, false, a.flags);
    if (active) {
        Ray r;
        make_ray(v, vi, vj, r);
        OctreeView o;
        o.nodes = reinterpret_cast<const ONode *>(oa.nodes);
        o.n_nodes = oa.n_nodes;
        o.verts = oa.verts;
        o.edges = oa.edges;
        o.edges_f = reinterpret_cast<const float4 *>(oa.edges_f);
        o.n_cells = oa.n_cells;
        o.depth = oa.depth;
        for (int i = 0; i < 3; i++) {
            o.dle[i] = oa.dle[i];
            o.dre[i] = oa.dre[i];
            o.size[i] = ytgb::dsub(oa.dre[i], oa.dle[i]);
        }
        unsigned long long th = MODE == MODE_TRACE ? hashes[p] : 0ull;
        long long tcount = 0;
        const bool ok = octree_ray<MODE, CTF>(a, o, s_tab, r, st, th, tcount);
        if (!ok) set_error(a.error, YTGB_DEVERR_STEP_LIMIT);
        if (MODE == MODE_TRACE) {
            hashes[p] = th;
            counts[p] += tcount;
        } else {
            for (int c = 0; c < 4; c++)
                if (st.touched & (1u << c)) img[c] = (double)st.xh[c] + (double)st.xl[c];
        }
    }
    if (a.counters) {
        if (st.visits) atomicAdd(&s_cnt[0], (unsigned long long)st.visits);
        if (st.walks) atomicAdd(&s_cnt[1], (unsigned long long)st.walks);
        if (st.guarded) atomicAdd(&s_cnt[3], (unsigned long long)st.guarded);
        if (active) atomicAdd(&s_cnt[2], 1ull);
        __syncthreads();
        if (tid < 4 && s_cnt[tid]) atomicAdd(a.counters + tid, s_cnt[tid]);
    }
}

int octree_checks(const ytgb_render_args *a, const ytgb_octree_args *o, bool trace, size_t *smem) {
    if (!a || !o) {
        ytgb_set_error("ytgb_render_octree: null arguments");
        return YTGB_ERR_INVALID;
    }
    const ytgb_view &v = a->view;
    if (v.nx <= 0 || v.ny <= 0 || (long long)v.nx * v.ny > (1ll << 40)) {
        ytgb_set_error("ytgb_render_octree: bad image size");
        return YTGB_ERR_INVALID;
    }
    if (v.lens != YTGB_LENS_PER_PIXEL && v.lens != YTGB_LENS_PERSPECTIVE) {
        ytgb_set_error("ytgb_render_octree: the octree path needs per-pixel rays (per-pixel or perspective lens)");
        return YTGB_ERR_INVALID;
    }
    if (v.lens == YTGB_LENS_PER_PIXEL && (!v.px_pos || !v.px_dir)) {
        ytgb_set_error("ytgb_render_octree: per-pixel lens needs px_pos / px_dir");
        return YTGB_ERR_INVALID;
    }
    if (!o->nodes || o->n_nodes <= 0 || o->n_cells < 0 || (o->n_cells > 0 && (!o->verts || !o->edges)) ||
        o->depth < 0 || o->depth > OCT_MAX_DEPTH) {
        ytgb_set_error("ytgb_render_octree: bad octree arguments (depth must be <= 30)");
        return YTGB_ERR_INVALID;
    }
    if (!trace && !a->image) {
        ytgb_set_error("ytgb_render_octree: missing image");
        return YTGB_ERR_INVALID;
    }
    if (a->kind < 0 || a->kind > 4 || a->n_samples < 1) {
        ytgb_set_error("ytgb_render_octree: bad sampler kind or n_samples");
        return YTGB_ERR_INVALID;
    }
    if (!trace && a->data != o->verts) {
        ytgb_set_error("ytgb_render_octree: args->data must be the octree's vertex array");
        return YTGB_ERR_INVALID;
    }
    auto mis = [](const void *q, uintptr_t al) { return q && ((uintptr_t)q & (al - 1)) != 0; };
    if (mis(o->nodes, 8) || mis(o->verts, 4) || mis(o->edges, 8) || mis(o->edges_f, 16) || mis(a->image, 8) || mis(a->tf_tables, 16) ||
        mis(a->counters, 8) || mis(a->error, 4) || mis(v.px_pos, 8) || mis(v.px_dir, 8) || mis(a->data_lo, 4)) {
        ytgb_set_error("ytgb_render_octree: misaligned pointer");
        return YTGB_ERR_INVALID;
    }
    *smem = 0;
    if (!trace && (a->kind == YTGB_VOLUME_RENDER || a->kind == YTGB_LIGHT_SOURCE)) {
        const ytgb_tf &t = a->tf;
        if (!a->tf_tables || t.n_fits < 0 || t.n_fits > 6 || t.nbins_max < 2 || t.nbins_max > YTGB_TF_MAX_BINS ||
            (t.ctf_fast && t.n_fits != 4)) {
            ytgb_set_error("ytgb_render_octree: bad transfer function");
            return YTGB_ERR_INVALID;
        }
        const bool ctf = a->kind == YTGB_VOLUME_RENDER && t.ctf_fast;
        *smem = ctf ? (size_t)3 * t.nbins_max * sizeof(float4) : (size_t)t.n_fits * t.nbins_max * sizeof(float4);
        if (*smem > 200 * 1024) {
            ytgb_set_error("ytgb_render_octree: transfer-function tables exceed 200 KB of shared memory");
            return YTGB_ERR_INVALID;
        }
    }
    return YTGB_OK;
}

template <int MODE, int CTF>
int octree_launch(const ytgb_render_args *a, const ytgb_octree_args *o, size_t smem, cudaStream_t s,
                  unsigned long long *h, long long *c) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(octree_kernel<MODE, CTF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) {
            ytgb_set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return YTGB_ERR_CUDA;
        }
    }
    const long long blocks = (long long)((a->view.nx + OTILE_X - 1) / OTILE_X) * ((a->view.ny + OTILE_Y - 1) / OTILE_Y);
    if (blocks > 0x7fffffffll) {
        ytgb_set_error("ytgb_render_octree: image too large");
        return YTGB_ERR_INVALID;
    }
    ytgb_render_args b = *a;
    view_derive(b.view);
    octree_kernel<MODE, CTF><<<(unsigned)blocks, OBLOCK, smem, s>>>(b, *o, h, c);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("octree launch: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return YTGB_OK;
}

}  // namespace

extern "C" int ytgb_render_octree(const ytgb_render_args *a, const ytgb_octree_args *o, void *stream) {
    size_t smem = 0;
    if (int st = octree_checks(a, o, false, &smem)) return st;
    cudaStream_t s = (cudaStream_t)stream;
    switch (a->kind) {
    case YTGB_VOLUME_RENDER:
        return a->tf.ctf_fast ? octree_launch<MODE_VR, 1>(a, o, smem, s, nullptr, nullptr)
                              : octree_launch<MODE_VR, 0>(a, o, smem, s, nullptr, nullptr);
    case YTGB_LIGHT_SOURCE: return octree_launch<MODE_LIGHT, 0>(a, o, smem, s, nullptr, nullptr);
    case YTGB_PROJECTION: return octree_launch<MODE_PROJ, 0>(a, o, 0, s, nullptr, nullptr);
    case YTGB_INTERPOLATED_PROJECTION: return octree_launch<MODE_IPROJ, 0>(a, o, 0, s, nullptr, nullptr);
    default: return octree_launch<MODE_MIP, 0>(a, o, 0, s, nullptr, nullptr);
    }
}

extern "C" int ytgb_trace_octree(const ytgb_render_args *a, const ytgb_octree_args *o, unsigned long long *hashes,
                                 long long *counts, void *stream) {
    size_t smem = 0;
    if (int st = octree_checks(a, o, true, &smem)) return st;
    if (!hashes || !counts || ((uintptr_t)hashes & 7) || ((uintptr_t)counts & 7)) {
        ytgb_set_error("ytgb_trace_octree: null or misaligned hash / count arrays");
        return YTGB_ERR_INVALID;
    }
    return octree_launch<MODE_TRACE, 0>(a, o, 0, (cudaStream_t)stream, hashes, counts);
}
