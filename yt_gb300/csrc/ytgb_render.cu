// ytgb_render.cu -- the per-pixel-ray sampler kernels of libytgb (sm_103a).
//
// One CUDA thread owns one pixel ray for the whole launch and walks every
// brick of the view in the kd viewpoint order, so the per-brick Python loop,
// OpenMP region and image read/write of yt's cast_through_kdtree
// (image_samplers.pyx:146-197) disappear.  Each warp bins the ordered brick
// list against its 32 pixels (the bricks' pixel rectangles) into a list in
// shared memory, so a ray only looks at bricks whose rectangle can contain
// it, and no warp waits for another.
//
// Precision split.  The cell walk of walk_volume (grid_traversal.pyx:26-140)
// is reproduced bit for bit: every float64 value the walk compares or hands
// to its sampler (intersect_t, tmax, tdelta, enter_t, exit_t, the cell index)
// is computed from the same operands in the same order as the reference, as
// _rn intrinsics (never contracted).  On GB300 the float64 pipe is far slower
// than float32, so everything else is kept off it:
//   * comparisons of walk values use order-preserving int64 keys;
//   * per cell `tmax += tdelta` runs as an integer add on the bit pattern
//     (float64 only when tmax leaves its binade) and `exit_t - enter_t` as
//     an integer difference converted to float32 once, by 32-bit integer
//     conversions (a 64-bit conversion runs on the float64 pipe);
//   * the sample position is tracked in float32, in cell-local coordinates
//     reset exactly on the axis the walk steps along;
//   * bricks a ray clearly misses, faces it clearly does not enter through,
//     and start points clearly outside a brick are rejected by float32 tests
//     whose margins exceed their float32 error by orders of magnitude, before
//     the exact float64 tests;
//   * the per-walk state is kept small (the rays themselves live in shared
//     memory, each ray keeps its tdelta products for the last brick's cell
//     width there, and the per-view constants of the perspective rays are
//     formed once on the host).
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
#include <cstring>
#include <mutex>
#include <string>

#include "ytgb.h"
#include "ytgb_internal.h"
#include "ytgb_ray.cuh"

namespace {

using namespace ytgb;

// Tile shapes (image rows vi x image columns vj per block); the autotuner
// picks one per workload class.  All shapes are 128 threads.
template <int TS> struct TileShape;
template <> struct TileShape<0> { static constexpr int X = 8, Y = 16; };
template <> struct TileShape<1> { static constexpr int X = 16, Y = 8; };
template <> struct TileShape<2> { static constexpr int X = 4, Y = 32; };
constexpr int BLOCK = 128;
constexpr int NWARP = BLOCK / 32;
// Resident blocks per SM the kernels are compiled for.  The per-ray walk is
// latency-bound (dependent integer and float64 steps), so warps per SM
// count for more than registers.  The single-view kernel takes 6 (80
// registers, a few spills in the per-walk state): on the 1024^2 AMR frame
// 1.199 ms against 1.234 ms at 5 (96 registers, no spills), and the
// projections 3-6 % faster.  The persistent batch kernel, whose loop keeps
// more state, takes 5: the 64-view batch runs 32.7 ms against 33.2 ms at
// 6.  The single-view kernel's float64-range-decision variants (V_REF, the
// served form's) keep 5 too: at 80 registers their rare float64 path
// spilled ~1 KB a thread and the served frame ran 2.46 ms against 2.03 ms
// at 96.  Images are identical at every setting.  YTGB_MIN_BLOCKS sets both
// (a second build at another budget, for the bit-identity test).
#ifdef YTGB_MIN_BLOCKS
constexpr int MIN_BLOCKS = YTGB_MIN_BLOCKS, BATCH_MIN_BLOCKS = YTGB_MIN_BLOCKS;
#else
constexpr int MIN_BLOCKS = 6, BATCH_MIN_BLOCKS = 5;
#endif

// Selected bricks a warp holds before walking them (flushed in order when
// nearly full).
constexpr int SEL_CAP = 128;

struct TileSmem {
    Ray ray[BLOCK];                // each thread's ray, read per brick walk instead of held in registers
    int sel[NWARP][SEL_CAP];       // each warp's selected order entries
};

// Stage the transfer function of a volume-rendering view in shared memory:
// the ColorTransferFunction layout repacked as y[4], dy[4], d0 per bin (one
// bin lookup serves all four tables), other table sets as they are.
template <int CTF>
__device__ __forceinline__ void stage_tf(const ytgb_render_args &a, float4 *s_tab) {
    const float4 *g = reinterpret_cast<const float4 *>(a.tf_tables);
    const int nb = a.tf.nbins_max;
    if (CTF) {
        for (int b = threadIdx.x; b < nb; b += BLOCK) {
            float4 t0 = __ldg(g + 0 * nb + b), t1 = __ldg(g + 1 * nb + b);
            float4 t2 = __ldg(g + 2 * nb + b), t3 = __ldg(g + 3 * nb + b);
            s_tab[3 * b + 0] = make_float4(t0.x, t1.x, t2.x, t3.x);
            s_tab[3 * b + 1] = make_float4(t0.y, t1.y, t2.y, t3.y);
            s_tab[3 * b + 2] = make_float4(t3.z, t3.w, 0.f, 0.f);
        }
    } else {
        const int n = a.tf.n_fits * nb;
        for (int k = threadIdx.x; k < n; k += BLOCK) s_tab[k] = __ldg(g + k);
    }
}

// One warp's 32 pixels of one tile of one view: cast_through_kdtree
// (image_samplers.pyx:146-197) for every brick of the view, restricted to
// these pixels.  The warp bins the ordered brick list against its pixels'
// rectangle 32 bricks at a time (one per lane: ballot and prefix count into
// the warp's list, order kept) and walks the list whenever it is nearly full
// and at the end; each ray walks the listed bricks whose pixel rectangle
// holds its pixel.  Nothing waits on other warps, so a warp whose rays end
// early takes its next work at once.
//   bx, by: the block tile (TX x TY pixels); w: which 32 of its 128 pixels;
//   tab: the transfer-function tables (shared: TG false; global: TG true);
//   slot: this thread's ray slot in sm.ray, wl: its warp's list in sm.sel.
template <int MODE, int VAR, int TS, bool TG>
__device__ __forceinline__ void warp_tile(const ytgb_render_args &a, int bx, int by, int w, const float4 *tab,
                                          TileSmem &sm, int slot, int wl, unsigned long long *hashes,
                                          long long *counts) {
    constexpr int TX = TileShape<TS>::X, TY = TileShape<TS>::Y;
    constexpr int WROWS = 32 / TY;  // image rows of a warp's pixels
    const ytgb_view &v = a.view;
    const int lane = threadIdx.x & 31;
    const int t = w * 32 + lane;  // the pixel within the block tile
    const int vj = by * TY + (t % TY);
    const int vi = bx * TX + (t / TY);
    const bool active = vi < v.nx && vj < v.ny;
    const int r0 = bx * TX + w * WROWS, r1 = r0 + WROWS;  // the warp's pixel rectangle
    const int c0 = by * TY, c1 = c0 + TY;
    const size_t p = active ? (size_t)vi * v.ny + vj : 0;

    Ray &r = sm.ray[slot];
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
    const int n_order = a.n_order;
    int *sel = sm.sel[wl];
    int nsel = 0;  // the same in every lane
    for (int base = 0; base < n_order; base += 32) {
        const int k = base + lane;
        bool hit = false;
        if (k < n_order) {
            const int4 rc = __ldg(rects + k);
            hit = rc.x < r1 && rc.y > r0 && rc.z < c1 && rc.w > c0;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (hit) sel[nsel + __popc(bal & ((1u << lane) - 1u))] = k;
        nsel += __popc(bal);
        if (nsel > SEL_CAP - 32 || base + 32 >= n_order) {
            __syncwarp();
            for (int j = 0; active && j < nsel; j++) {
                const int kk = sel[j];
                const int4 rc = __ldg(rects + kk);
                if (vi < rc.x || vi >= rc.y || vj < rc.z || vj >= rc.w) continue;
                walk_brick<MODE, VAR, TG>(a, tab, r, __ldg(a.order + kk), st);
            }
            __syncwarp();  // the list is rewritten by the next passes
            nsel = 0;
        }
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
        // per warp: one sum per counter, one atomic per counter
        const unsigned sv = __reduce_add_sync(0xffffffffu, st.visits);
        const unsigned sw = __reduce_add_sync(0xffffffffu, st.walks);
        const unsigned sg = __reduce_add_sync(0xffffffffu, st.guarded);
        const unsigned sr = __popc(__ballot_sync(0xffffffffu, active));
        if (lane == 0) {
            if (sv) atomicAdd(a.counters + 0, (unsigned long long)sv);
            if (sw) atomicAdd(a.counters + 1, (unsigned long long)sw);
            if (sr) atomicAdd(a.counters + 2, (unsigned long long)sr);
            if (sg) atomicAdd(a.counters + 3, (unsigned long long)sg);
        }
    }
}

// One view, one tile per block (four warps of 32 pixels).
template <int MODE, int VAR, int TS>
__global__ void __launch_bounds__(BLOCK, (VAR & V_REF) ? BATCH_MIN_BLOCKS : MIN_BLOCKS) render_kernel(const ytgb_render_args a, unsigned long long *hashes,
                                                       long long *counts) {
    extern __shared__ float4 s_tab[];
    __shared__ TileSmem sm;
    if (MODE == MODE_VR || MODE == MODE_LIGHT) {
        stage_tf<VAR & V_CTF>(a, s_tab);
        __syncthreads();
    }
    const int w = threadIdx.x >> 5;
    warp_tile<MODE, VAR, TS, false>(a, blockIdx.y, blockIdx.x, w, s_tab, sm, threadIdx.x, w, hashes, counts);
}

// Many views in one persistent launch: every warp pulls work items -- one
// warp's 32 pixels of a (view, tile) -- from a device counter until the
// batch is drained, so small and large views share the GPU without a launch
// per view and no warp waits for another.  An item's view is found by binary
// search over the entries' first tiles.  STAGED: every entry uses the same
// transfer-function tables (ytgb_batch_plan asks for shared memory only
// then), staged once per block like render_kernel's; otherwise the views may
// use different tables and read them from global memory (cached).  Every
// loop iteration takes a new item: a warp runs at most as many iterations as
// there are items (no spin, and no barrier after the staging).
template <int MODE, int VAR, int TS, bool STAGED>
__global__ void __launch_bounds__(BLOCK, BATCH_MIN_BLOCKS) batch_kernel(const ytgb_batch_entry *entries, int n_entries,
                                                      int total_tiles, int *queue) {
    extern __shared__ float4 s_tab[];
    __shared__ TileSmem sm;
    if (STAGED) {
        // the launch's dynamic shared memory must hold the tables (a device
        // table cannot be checked on the host): too little is an error, not
        // a write out of bounds
        unsigned dyn = 0;
        asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
        const ytgb_render_args &a0 = entries[0].args;
        const size_t need = (size_t)((VAR & V_CTF) ? 3 : a0.tf.n_fits) * a0.tf.nbins_max * sizeof(float4);
        if (need > dyn) {
            if (threadIdx.x == 0) set_error(a0.error, YTGB_DEVERR_BAD_TF);
            return;
        }
        stage_tf<VAR & V_CTF>(a0, s_tab);
        __syncthreads();
    }
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const long long total_items = (long long)total_tiles * NWARP;
    while (true) {
        int item = 0;
        if (lane == 0) item = atomicAdd(queue, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item < 0 || item >= total_items) break;
        const int tile = item / NWARP;
        int lo = 0, hi = n_entries - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&entries[mid].tile_begin) <= tile) lo = mid;
            else hi = mid - 1;
        }
        const ytgb_batch_entry &e = entries[lo];
        const int t = tile - __ldg(&e.tile_begin);
        const int ty = __ldg(&e.tiles_y);
        const float4 *tab = STAGED ? s_tab : reinterpret_cast<const float4 *>(e.args.tf_tables);
        warp_tile<MODE, VAR, TS, !STAGED>(e.args, t / ty, t % ty, item % NWARP, tab, sm, threadIdx.x, wl, nullptr,
                                         nullptr);
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
    if (a->kind < 0 || a->kind > 4) {
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
    if (v.lens != YTGB_LENS_PER_PIXEL && v.lens != YTGB_LENS_PLANE_PARALLEL && v.lens != YTGB_LENS_PERSPECTIVE) {
        ytgb_set_error("ytgb_render: unknown lens");
        return YTGB_ERR_INVALID;
    }
    if (a->n_samples < 1) {
        ytgb_set_error("ytgb_render: n_samples must be >= 1");
        return YTGB_ERR_INVALID;
    }
    if (!(a->range_eps >= 0.0f) || !(a->range_eps <= 3.0e38f)) {
        ytgb_set_error("ytgb_render: range_eps must be finite and >= 0");
        return YTGB_ERR_INVALID;
    }
    // the kernels load these with vector / 8-byte accesses
    auto misaligned = [](const void *p, uintptr_t al) { return p && ((uintptr_t)p & (al - 1)) != 0; };
    if (misaligned(a->rects, 16) || misaligned(a->tf_tables, 16) || misaligned(a->bricks, 16) ||
        misaligned(a->bounds, 8) || misaligned(a->image, 8) || misaligned(a->zbuffer, 8) ||
        misaligned(a->counters, 8) || misaligned(v.px_pos, 8) || misaligned(v.px_dir, 8) ||
        misaligned(a->order, 4) || misaligned(a->data, 4) || misaligned(a->error, 4) ||
        misaligned(a->data_lo, 4)) {
        ytgb_set_error("ytgb_render: misaligned pointer (rects, tf_tables and bricks need 16 bytes, "
                       "float64 arrays 8)");
        return YTGB_ERR_INVALID;
    }
    if (a->n_order > 0 && !a->bounds) {
        ytgb_set_error("ytgb_render: missing cell-boundary tables");
        return YTGB_ERR_INVALID;
    }
    if (!trace && (a->kind == YTGB_VOLUME_RENDER || a->kind == YTGB_LIGHT_SOURCE) && !a->tf_tables) {
        ytgb_set_error("ytgb_render: volume rendering needs a transfer function");
        return YTGB_ERR_INVALID;
    }
    return YTGB_OK;
}

// Whether two launches read the same transfer function: the same packed
// tables and an identical header.
bool same_tf(const ytgb_render_args &a, const ytgb_render_args &b) {
    return a.tf_tables == b.tf_tables && std::memcmp(&a.tf, &b.tf, sizeof(ytgb_tf)) == 0;
}

// Transfer-function header checks and the shared-memory bytes its tables take
// (in the packed ColorTransferFunction layout when ctf_layout).
int tf_check(const ytgb_tf &t, size_t *smem, bool ctf_layout) {
    if (t.n_fits < 0 || t.n_fits > 6 || t.nbins_max < 2 || t.nbins_max > YTGB_TF_MAX_BINS) {
        ytgb_set_error("inconsistent transfer function header");
        return YTGB_ERR_INVALID;
    }
    for (int q = 0; q < t.n_fits; q++) {
        if (t.nbins[q] < 2 || t.nbins[q] > t.nbins_max || t.field_id[q] < 0 || t.field_id[q] > 5 ||
            t.weight_field_id[q] < -1 || t.weight_field_id[q] > 5 || t.weight_table_id[q] < -1 ||
            t.weight_table_id[q] >= t.n_fits) {
            ytgb_set_error("transfer function table ids out of range");
            return YTGB_ERR_INVALID;
        }
    }
    for (int c = 0; c < 6; c++) {
        if (t.field_table_ids[c] < 0 || t.field_table_ids[c] > 5) {
            ytgb_set_error("field_table_ids out of range");
            return YTGB_ERR_INVALID;
        }
    }
    if (t.ctf_fast && (t.n_fits != 4 || t.nbins[0] != t.nbins_max)) {
        ytgb_set_error("ctf_fast set on tables that are not a ColorTransferFunction");
        return YTGB_ERR_INVALID;
    }
    *smem = ctf_layout ? (size_t)3 * t.nbins_max * sizeof(float4) : (size_t)t.n_fits * t.nbins_max * sizeof(float4);
    if (*smem > 200 * 1024) {
        ytgb_set_error("transfer-function tables exceed 200 KB of shared memory");
        return YTGB_ERR_INVALID;
    }
    return YTGB_OK;
}

template <typename K>
int set_smem(K kernel, size_t smem) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) {
            ytgb_set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return YTGB_ERR_CUDA;
        }
    }
    return YTGB_OK;
}

int launch_status(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ytgb_set_error(std::string(what) + ": " + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return YTGB_OK;
}

template <int MODE, int VAR, int TS>
int launch(const ytgb_render_args *a, size_t smem, cudaStream_t s, unsigned long long *h, long long *c) {
    constexpr int TX = TileShape<TS>::X, TY = TileShape<TS>::Y;
    dim3 grid((a->view.ny + TY - 1) / TY, (a->view.nx + TX - 1) / TX);
    if (grid.y > 65535) {
        ytgb_set_error("ytgb_render: image too tall");
        return YTGB_ERR_INVALID;
    }
    if (int st = set_smem(render_kernel<MODE, VAR, TS>, smem)) return st;
    ytgb_render_args b = *a;
    view_derive(b.view);
    render_kernel<MODE, VAR, TS><<<grid, BLOCK, smem, s>>>(b, h, c);
    return launch_status("render launch");
}

template <int MODE, int VAR>
int launch_ts(int ts, const ytgb_render_args *a, size_t smem, cudaStream_t s, unsigned long long *h, long long *c) {
    switch (ts) {
    case 1: return launch<MODE, VAR, 1>(a, smem, s, h, c);
    case 2: return launch<MODE, VAR, 2>(a, smem, s, h, c);
    default: return launch<MODE, VAR, 0>(a, smem, s, h, c);
    }
}

int tile_shape_of(uint32_t flags) { return (int)((flags >> YTGB_FLAG_TILE_SHIFT) & 0xfu); }

template <int MODE>
int launch_var(int var, int ts, const ytgb_render_args *a, size_t smem, cudaStream_t s) {
    switch (var) {
    case V_CTF: return launch_ts<MODE, V_CTF>(ts, a, smem, s, nullptr, nullptr);
    case V_REF: return launch_ts<MODE, V_REF>(ts, a, smem, s, nullptr, nullptr);
    case V_CTF | V_REF: return launch_ts<MODE, V_CTF | V_REF>(ts, a, smem, s, nullptr, nullptr);
    default: return launch_ts<MODE, 0>(ts, a, smem, s, nullptr, nullptr);
    }
}

template <int MODE, int VAR, int TS>
int batch_launch_t(const ytgb_batch_entry *d, int n, int total, int *queue, int blocks, size_t smem,
                   cudaStream_t s) {
    // smem > 0: every entry shares the transfer function (ytgb_batch_plan),
    // staged in shared memory; 0: tables read from global memory
    const bool staged = smem > 0 && (MODE == MODE_VR || MODE == MODE_LIGHT);
    auto kernel = staged ? batch_kernel<MODE, VAR, TS, true> : batch_kernel<MODE, VAR, TS, false>;
    if (!staged) smem = 0;
    if (int st = set_smem(kernel, smem)) return st;
    if (blocks <= 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, BLOCK, smem);
        blocks = sms * (per_sm > 0 ? per_sm : 1);
    }
    if (blocks > total) blocks = total;
    if (blocks < 1) blocks = 1;
    kernel<<<blocks, BLOCK, smem, s>>>(d, n, total, queue);
    return launch_status("batch launch");
}

template <int MODE, int VAR>
int batch_launch_ts(int ts, const ytgb_batch_entry *d, int n, int total, int *queue, int blocks, size_t smem,
                    cudaStream_t s) {
    switch (ts) {
    case 1: return batch_launch_t<MODE, VAR, 1>(d, n, total, queue, blocks, smem, s);
    case 2: return batch_launch_t<MODE, VAR, 2>(d, n, total, queue, blocks, smem, s);
    default: return batch_launch_t<MODE, VAR, 0>(d, n, total, queue, blocks, smem, s);
    }
}

}  // namespace

extern "C" int ytgb_render(const ytgb_render_args *a, void *stream) {
    int st = check_args(a, false);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const int ts = tile_shape_of(a->flags);
    if (ts > 2) {
        ytgb_set_error("ytgb_render: unknown tile shape");
        return YTGB_ERR_INVALID;
    }
    const int var = render_variant(*a);
    if (a->kind == YTGB_LIGHT_SOURCE) {
        size_t smem = 0;
        if ((st = tf_check(a->tf, &smem, false))) return st;
        return (var & V_REF) ? launch_ts<MODE_LIGHT, V_REF>(ts, a, smem, s, nullptr, nullptr)
                             : launch_ts<MODE_LIGHT, 0>(ts, a, smem, s, nullptr, nullptr);
    }
    if (a->kind == YTGB_VOLUME_RENDER) {
        size_t smem = 0;
        if ((st = tf_check(a->tf, &smem, a->tf.ctf_fast != 0))) return st;
        return launch_var<MODE_VR>(var, ts, a, smem, s);
    }
    switch (a->kind) {
    case YTGB_PROJECTION: return launch_ts<MODE_PROJ, 0>(ts, a, 0, s, nullptr, nullptr);
    case YTGB_INTERPOLATED_PROJECTION: return launch_ts<MODE_IPROJ, 0>(ts, a, 0, s, nullptr, nullptr);
    default: return launch_ts<MODE_MIP, 0>(ts, a, 0, s, nullptr, nullptr);
    }
}

extern "C" int ytgb_trace(const ytgb_render_args *a, unsigned long long *hashes, long long *counts, void *stream) {
    int st = check_args(a, true);
    if (st) return st;
    if (!hashes || !counts) {
        ytgb_set_error("ytgb_trace: null hash / count arrays");
        return YTGB_ERR_INVALID;
    }
    return launch<MODE_TRACE, 0, 0>(a, 0, (cudaStream_t)stream, hashes, counts);
}

extern "C" int ytgb_batch_plan(ytgb_batch_entry *entries, int32_t n, int32_t tile_shape, int32_t *total_tiles,
                               int32_t *smem_bytes) {
    if (!entries || n <= 0 || !total_tiles || !smem_bytes || tile_shape < 0 || tile_shape > 2) {
        ytgb_set_error("ytgb_batch_plan: bad arguments");
        return YTGB_ERR_INVALID;
    }
    const int TX = tile_shape == 1 ? 16 : (tile_shape == 2 ? 4 : 8);
    const int TY = BLOCK / TX;
    const int kind = entries[0].args.kind;
    const int var = render_variant(entries[0].args);
    const int ctf = var & V_CTF;
    long long total = 0;
    size_t smem = 0;
    bool shared_tf = true;
    for (int32_t k = 0; k < n; k++) {
        ytgb_render_args &a = entries[k].args;
        if (int st = check_args(&a, false)) return st;
        view_derive(a.view);
        if (a.kind != kind || render_variant(a) != var) {
            ytgb_set_error("ytgb_batch_plan: every entry of a batch must use the same sampler, table layout and "
                           "range decisions (data_lo with range_eps > 0, or neither)");
            return YTGB_ERR_INVALID;
        }
        shared_tf = shared_tf && same_tf(a, entries[0].args);
        if (kind == YTGB_VOLUME_RENDER || kind == YTGB_LIGHT_SOURCE) {
            size_t sm = 0;
            if (int st = tf_check(a.tf, &sm, kind == YTGB_VOLUME_RENDER && ctf != 0)) return st;
            smem = sm > smem ? sm : smem;
        }
        const int tx = (a.view.nx + TX - 1) / TX, ty = (a.view.ny + TY - 1) / TY;
        entries[k].tile_begin = (int32_t)total;
        entries[k].tiles_y = ty;
        entries[k].tiles = tx * ty;
        total += (long long)tx * ty;
        if (total * NWARP > 0x7fff0000LL) {  // warp work items count in an int32
            ytgb_set_error("ytgb_batch_plan: too many tiles");
            return YTGB_ERR_INVALID;
        }
    }
    *total_tiles = (int32_t)total;
    *smem_bytes = shared_tf ? (int32_t)smem : 0;
    return YTGB_OK;
}

// A batch launch of one sampler kind and variant (YTGB_VARIANT_* bits, the
// kernels' V_CTF / V_REF).
static_assert(YTGB_VARIANT_CTF == V_CTF && YTGB_VARIANT_RANGE64 == V_REF, "variant bits");
static int batch_dispatch(int32_t kind, int32_t variant, int32_t tile_shape, const ytgb_batch_entry *entries, int32_t n,
                   int32_t total_tiles, int32_t *queue, int32_t blocks, size_t smem, cudaStream_t s) {
    const bool ref = (variant & YTGB_VARIANT_RANGE64) != 0;
    switch (kind) {
    case YTGB_VOLUME_RENDER:
        if (variant & YTGB_VARIANT_CTF)
            return ref ? batch_launch_ts<MODE_VR, V_CTF | V_REF>(tile_shape, entries, n, total_tiles, queue, blocks,
                                                                 smem, s)
                       : batch_launch_ts<MODE_VR, V_CTF>(tile_shape, entries, n, total_tiles, queue, blocks, smem, s);
        return ref ? batch_launch_ts<MODE_VR, V_REF>(tile_shape, entries, n, total_tiles, queue, blocks, smem, s)
                   : batch_launch_ts<MODE_VR, 0>(tile_shape, entries, n, total_tiles, queue, blocks, smem, s);
    case YTGB_LIGHT_SOURCE:
        return ref ? batch_launch_ts<MODE_LIGHT, V_REF>(tile_shape, entries, n, total_tiles, queue, blocks, smem, s)
                   : batch_launch_ts<MODE_LIGHT, 0>(tile_shape, entries, n, total_tiles, queue, blocks, smem, s);
    case YTGB_PROJECTION:
        return batch_launch_ts<MODE_PROJ, 0>(tile_shape, entries, n, total_tiles, queue, blocks, 0, s);
    case YTGB_INTERPOLATED_PROJECTION:
        return batch_launch_ts<MODE_IPROJ, 0>(tile_shape, entries, n, total_tiles, queue, blocks, 0, s);
    default:
        return batch_launch_ts<MODE_MIP, 0>(tile_shape, entries, n, total_tiles, queue, blocks, 0, s);
    }
}

extern "C" int ytgb_batch_render(const ytgb_batch_entry *d_entries, int32_t n, int32_t kind, int32_t variant,
                                 int32_t tile_shape, int32_t total_tiles, int32_t smem_bytes, int32_t *d_queue,
                                 int32_t blocks, void *stream) {
    if (!d_entries || n <= 0 || total_tiles <= 0 || !d_queue || tile_shape < 0 || tile_shape > 2 || kind < 0 ||
        kind > 4 || smem_bytes < 0 || smem_bytes > 200 * 1024 || ((uintptr_t)d_entries & 15) != 0 ||
        ((uintptr_t)d_queue & 3) != 0 || variant < 0 || variant > 3) {
        ytgb_set_error("ytgb_batch_render: bad arguments");
        return YTGB_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(d_queue, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("ytgb_batch_render: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return batch_dispatch(kind, variant, tile_shape, d_entries, n, total_tiles, d_queue, blocks,
                          (size_t)smem_bytes, s);
}

// ---- ytgb_batch_render_noalloc: the persistent batch with static scratch --
//
// ytgb_batch_render needs two device buffers from its caller: the planned
// entry table and the work-queue counter.  Some callers cannot allocate
// them.  cudaMalloc and cudaFree synchronise the whole device, which a
// serving loop overlapping renders with other work cannot afford per call;
// a process whose device memory is already reserved by another allocator
// (a framework's caching pool) can see a raw cudaMalloc fail; and a caller
// that holds only host data and pointers it was given (a binding that
// forwards yt's samplers) has no device allocator to call.  This variant
// keeps both buffers in a fixed region of static device memory instead, so
// the call allocates nothing.
//
// Layout of the region: the work-queue counter in the first 256 bytes, then
// up to YTGB_NOALLOC_MAX_ENTRIES entries.  The counter must be zero when the
// kernel starts; every call clears it on its stream before the launch and
// overwrites the entries it uses, so nothing has to be zero beforehand.
// There is one region per device, so calls whose work overlaps on the
// device (two streams, or two host threads, with launches in flight at the
// same time) would overwrite each other's table and share one counter:
// callers must order them (one stream, or wait for one call's work before
// issuing the next).
constexpr size_t NOALLOC_QUEUE_BYTES = 256;
static __device__ __align__(256) unsigned char
    g_noalloc_scratch[NOALLOC_QUEUE_BYTES + (size_t)YTGB_NOALLOC_MAX_ENTRIES * sizeof(ytgb_batch_entry)];

namespace {
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// The region's device address, looked up once per device with that device
// current (the first call on a device does it).  cudaDeviceReset unloads
// the module with the device's primary context; the address cached here is
// then stale, so a process that resets a device does not call this entry
// point on it again (stated in ytgb.h).
int noalloc_scratch(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("ytgb_batch_render_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        ytgb_set_error("ytgb_batch_render_noalloc: device ordinal out of range");
        return YTGB_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            ytgb_set_error(std::string("ytgb_batch_render_noalloc: cudaGetSymbolAddress: ") +
                           cudaGetErrorString(e));
            return YTGB_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return YTGB_OK;
}


// The host copy of a planned batch against the launch arguments: every
// entry's arguments valid and of this sampler kind and table layout, the
// shared memory enough for every entry's tables, and the tile numbering the
// one ytgb_batch_plan writes for this tile shape.  The kernel stages each
// entry's tables into smem_bytes of shared memory and maps work items to
// tiles by this numbering, so a mismatch would write out of bounds or
// mis-tile an image; with the table on the host it is checked for free.
int noalloc_check_plan(const ytgb_batch_entry *h, int32_t n, int32_t kind, int32_t variant, int32_t tile_shape,
                       int32_t total_tiles, int32_t smem_bytes) {
    const int TX = tile_shape == 1 ? 16 : (tile_shape == 2 ? 4 : 8);
    const int TY = BLOCK / TX;
    long long total = 0;
    size_t smem = 0;
    bool shared_tf = true;
    for (int32_t k = 0; k < n; k++) {
        const ytgb_render_args &a = h[k].args;
        shared_tf = shared_tf && same_tf(a, h[0].args);
        if (int st = check_args(&a, false)) return st;
        if (a.kind != kind || render_variant(a) != variant) {
            ytgb_set_error("ytgb_batch_render_noalloc: entry " + std::to_string(k) +
                           " is not of the launch's sampler kind / variant");
            return YTGB_ERR_INVALID;
        }
        if (kind == YTGB_VOLUME_RENDER || kind == YTGB_LIGHT_SOURCE) {
            size_t sm = 0;
            if (int st = tf_check(a.tf, &sm, kind == YTGB_VOLUME_RENDER && (variant & V_CTF) != 0)) return st;
            smem = sm > smem ? sm : smem;
        }
        const long long tx = (a.view.nx + TX - 1) / TX, ty = (a.view.ny + TY - 1) / TY;
        ytgb_view dv = a.view;
        view_derive(dv);
        if (std::memcmp(&dv, &a.view, sizeof(dv)) != 0) {
            ytgb_set_error("ytgb_batch_render_noalloc: entry " + std::to_string(k) +
                           " has no derived view constants (run ytgb_batch_plan on the table)");
            return YTGB_ERR_INVALID;
        }
        if (h[k].tile_begin != total || h[k].tiles_y != ty || h[k].tiles != tx * ty) {
            ytgb_set_error("ytgb_batch_render_noalloc: entry " + std::to_string(k) +
                           " is not planned for this tile shape (run ytgb_batch_plan with it)");
            return YTGB_ERR_INVALID;
        }
        total += tx * ty;
    }
    if (total != total_tiles) {
        ytgb_set_error("ytgb_batch_render_noalloc: total_tiles does not match the planned entries");
        return YTGB_ERR_INVALID;
    }
    if (smem_bytes > 0 && (kind == YTGB_VOLUME_RENDER || kind == YTGB_LIGHT_SOURCE) &&
        (!shared_tf || (size_t)smem_bytes < smem)) {
        ytgb_set_error(shared_tf ? "ytgb_batch_render_noalloc: smem_bytes is below what the entries' tables take"
                                 : "ytgb_batch_render_noalloc: smem_bytes > 0 stages one transfer function, but "
                                   "the entries use different ones");
        return YTGB_ERR_INVALID;
    }
    return YTGB_OK;
}
}  // namespace

extern "C" int ytgb_batch_render_noalloc(const ytgb_batch_entry *h_entries, int32_t n, int32_t kind,
                                         int32_t variant, int32_t tile_shape, int32_t total_tiles,
                                         int32_t smem_bytes, int32_t blocks, void *stream) {
    if (n > YTGB_NOALLOC_MAX_ENTRIES) {
        ytgb_set_error("ytgb_batch_render_noalloc: " + std::to_string(n) + " entries exceed the static scratch (" +
                       std::to_string(YTGB_NOALLOC_MAX_ENTRIES) +
                       " views); split the batch or use ytgb_batch_render with a caller-allocated table");
        return YTGB_ERR_INVALID;
    }
    if (!h_entries || n <= 0 || total_tiles <= 0 || tile_shape < 0 || tile_shape > 2 || kind < 0 || kind > 4 ||
        smem_bytes < 0 || smem_bytes > 200 * 1024 || variant < 0 || variant > 3) {
        ytgb_set_error("ytgb_batch_render_noalloc: bad arguments");
        return YTGB_ERR_INVALID;
    }
    if (int st = noalloc_check_plan(h_entries, n, kind, variant, tile_shape, total_tiles, smem_bytes)) return st;
    unsigned char *base = nullptr;
    if (int st = noalloc_scratch(&base)) return st;
    int32_t *queue = reinterpret_cast<int32_t *>(base);
    ytgb_batch_entry *entries = reinterpret_cast<ytgb_batch_entry *>(base + NOALLOC_QUEUE_BYTES);
    cudaStream_t s = (cudaStream_t)stream;
    // A copy from pageable host memory is staged before cudaMemcpyAsync
    // returns, so such a table may be reused at once; a page-locked table
    // is read by the copy engine in stream order and must stay unchanged
    // until the stream has passed this call (stated in ytgb.h).
    cudaError_t e = cudaMemcpyAsync(entries, h_entries, (size_t)n * sizeof(ytgb_batch_entry),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("ytgb_batch_render_noalloc: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return batch_dispatch(kind, variant, tile_shape, entries, n, total_tiles, queue, blocks, (size_t)smem_bytes, s);
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
