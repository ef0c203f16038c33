// ytgb_prep.cu -- device brick preparation (vertex centring, log10, slicing).
//
// Replaces the host loop of yt's AMRKDTree.get_brick_data
// (amr_kdtree.py:325-374) over every kd leaf: one block per brick computes
// the brick's (dims+1)^3 vertex values from its grid's cell data
// (ytgb_vertex.cuh), applies log10 where requested and writes them as
// float32 into the brick's slot of the arena.  Every index the kernel forms
// is checked against the sizes it is given; a brick that does not fit its
// grid or the arena is skipped and reported through the error word.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <string>

#include "ytgb.h"
#include "ytgb_internal.h"
#include "ytgb_vertex.cuh"

namespace {

using namespace ytgb;

constexpr int PREP_BLOCK = 256;

__global__ void __launch_bounds__(PREP_BLOCK)
vertex_bricks_kernel(const double *cells, int64_t n_cells, const int64_t *grid_offset, const int32_t *grid_dims,
                     int32_t n_grids, const int32_t *brick_grid, const int32_t *brick_lo, const ytgb_brick *bricks,
                     int32_t field, int32_t log_field, float *arena, int64_t arena_len, int32_t *error,
                     float *arena_lo) {
    const int b = blockIdx.x;
    const int g = brick_grid[b];
    if (g < 0 || g >= n_grids) {
        if (threadIdx.x == 0) set_error(error, YTGB_DEVERR_BAD_BRICK);
        return;
    }
    const int n0 = grid_dims[3 * g], n1 = grid_dims[3 * g + 1], n2 = grid_dims[3 * g + 2];
    const int l0 = brick_lo[3 * b], l1 = brick_lo[3 * b + 1], l2 = brick_lo[3 * b + 2];
    const ytgb_brick &bk = bricks[b];
    const int d0 = bk.dims[0], d1 = bk.dims[1], d2 = bk.dims[2];
    const long long go = grid_offset[g];
    const long long nv = (long long)(d0 + 1) * (d1 + 1) * (d2 + 1);
    const long long out0 = bk.data_offset + (long long)field * bk.field_stride;
    // the leaf's vertices [l, l + d] must be vertices of the grid [0, n], the
    // grid's cells must lie in the cell array, and the slot in the arena
    const bool ok = n0 >= 2 && n1 >= 2 && n2 >= 2 && d0 > 0 && d1 > 0 && d2 > 0 && l0 >= 0 && l1 >= 0 &&
                    l2 >= 0 && l0 + d0 <= n0 && l1 + d1 <= n1 && l2 + d2 <= n2 && go >= 0 &&
                    go + (long long)n0 * n1 * n2 <= n_cells && field >= 0 && field < bk.n_fields && out0 >= 0 &&
                    out0 + nv <= arena_len && nv <= bk.field_stride;
    if (!ok) {
        if (threadIdx.x == 0) set_error(error, YTGB_DEVERR_BAD_BRICK);
        return;
    }
    const double *c = cells + go;
    float *out = arena + out0;
    const int e1 = d1 + 1, e2 = d2 + 1;
    for (long long t = threadIdx.x; t < nv; t += PREP_BLOCK) {
        const int k = (int)(t % e2);
        const long long r = t / e2;
        const int j = (int)(r % e1);
        const int i = (int)(r / e1);
        double v = vertex_value(c, n0, n1, n2, l0 + i, l1 + j, l2 + k);
        if (log_field) v = v <= 0.0 ? nan("") : log10(v);
        const float h = (float)v;
        out[t] = h;
        if (arena_lo) {
            const double err = v - (double)h;
            arena_lo[out0 + t] = isfinite(err) ? (float)err : 0.0f;
        }
    }
}

constexpr int GATHER_BLOCK = 256;

// One block per field (grid-stride over the fields): host float64 values,
// read over the CPU-GPU link, to float32 (and low parts) in the arena.
__global__ void __launch_bounds__(GATHER_BLOCK)
gather_fields_kernel(const double *const *src, const int64_t *count, const int64_t *dst_offset, int64_t n,
                     float *arena, float *arena_lo) {
    for (int64_t k = blockIdx.x; k < n; k += gridDim.x) {
        const double *s = src[k];
        const int64_t c = count[k];
        float *d = arena + dst_offset[k];
        float *dl = arena_lo ? arena_lo + dst_offset[k] : nullptr;
        for (int64_t i = threadIdx.x; i < c; i += GATHER_BLOCK) {
            const double v = s[i];
            const float h = (float)v;
            d[i] = h;
            if (dl) {
                const double r = v - (double)h;
                dl[i] = r == r && r - r == 0.0 ? (float)r : 0.0f;
            }
        }
    }
}

// One block per mask (grid-stride): the host uint8 cell mask into the mask
// arena; a brick with any byte other than 1 gets its mask_offset (it stays
// -1, "all ones", otherwise: VolumeRenderSampler samples a cell when its
// mask byte is 1, image_samplers.pyx:467-470).
__global__ void __launch_bounds__(GATHER_BLOCK)
gather_masks_kernel(const uint8_t *const *src, const int64_t *count, const int64_t *dst_offset, const int32_t *brick,
                    int64_t n, uint8_t *masks, ytgb_brick *desc) {
    for (int64_t k = blockIdx.x; k < n; k += gridDim.x) {
        const uint8_t *s = src[k];
        const int64_t c = count[k];
        uint8_t *d = masks + dst_offset[k];
        int other = 0;
        // 16-byte reads over the link where the source allows (one request
        // per warp moves 512 bytes instead of 32): the bytes before the first
        // 16-byte boundary, the whole vectors, then the rest
        const int64_t head = min(c, (int64_t)((16 - ((uintptr_t)s & 15)) & 15));
        const int64_t nvec = (c - head) >> 4;
        for (int64_t i = threadIdx.x; i < head; i += GATHER_BLOCK) {
            const uint8_t v = s[i];
            d[i] = v;
            other |= v != 1;
        }
        const uint4 *sv = reinterpret_cast<const uint4 *>(s + head);
        uint8_t *dv = d + head;
        const bool dst16 = ((uintptr_t)dv & 15) == 0;
        for (int64_t i = threadIdx.x; i < nvec; i += GATHER_BLOCK) {
            const uint4 w = sv[i];
            other |= (w.x != 0x01010101u) | (w.y != 0x01010101u) | (w.z != 0x01010101u) | (w.w != 0x01010101u);
            if (dst16) {
                reinterpret_cast<uint4 *>(dv)[i] = w;
            } else {
                const uint32_t wd[4] = {w.x, w.y, w.z, w.w};
                for (int b = 0; b < 16; b++) dv[16 * i + b] = (uint8_t)(wd[b >> 2] >> (8 * (b & 3)));
            }
        }
        for (int64_t i = head + (nvec << 4) + threadIdx.x; i < c; i += GATHER_BLOCK) {
            const uint8_t v = s[i];
            d[i] = v;
            other |= v != 1;
        }
        if (__syncthreads_or(other) && threadIdx.x == 0) desc[brick[k]].mask_offset = dst_offset[k];
    }
}

bool device_reads_host() {
    int dev = 0, pma = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) return false;
    return pma != 0;
}

}  // namespace

extern "C" int ytgb_device_reads_host(int32_t *out) {
    if (!out) {
        ytgb_set_error("ytgb_device_reads_host: null out");
        return YTGB_ERR_INVALID;
    }
    *out = device_reads_host() ? 1 : 0;
    return YTGB_OK;
}

extern "C" int ytgb_gather_fields(const double *const *src, const int64_t *count, const int64_t *dst_offset,
                                  int64_t n, float *d_arena, float *d_arena_lo, int64_t arena_len, void *stream) {
    if (n < 0 || arena_len < 0 || (n > 0 && (!src || !count || !dst_offset || !d_arena))) {
        ytgb_set_error("ytgb_gather_fields: bad arguments");
        return YTGB_ERR_INVALID;
    }
    if (n == 0) return YTGB_OK;
    if (!device_reads_host()) {
        ytgb_set_error("ytgb_gather_fields: the device cannot read pageable host memory");
        return YTGB_ERR_INVALID;
    }
    if (((uintptr_t)d_arena & 3) || ((uintptr_t)d_arena_lo & 3)) {
        ytgb_set_error("ytgb_gather_fields: misaligned arena");
        return YTGB_ERR_INVALID;
    }
    for (int64_t k = 0; k < n; k++) {
        if (count[k] < 0 || (count[k] > 0 && (!src[k] || ((uintptr_t)src[k] & 7))) || dst_offset[k] < 0 ||
            dst_offset[k] > arena_len - count[k]) {
            ytgb_set_error("ytgb_gather_fields: field " + std::to_string(k) + " is null, misaligned or does not "
                           "fit the arena");
            return YTGB_ERR_INVALID;
        }
    }
    const int blocks = (int)(n < 152 * 16 ? n : 152 * 16);
    gather_fields_kernel<<<blocks, GATHER_BLOCK, 0, (cudaStream_t)stream>>>(src, count, dst_offset, n, d_arena,
                                                                           d_arena_lo);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("ytgb_gather_fields: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return YTGB_OK;
}

extern "C" int ytgb_gather_masks(const uint8_t *const *src, const int64_t *count, const int64_t *dst_offset,
                                 const int32_t *brick, int64_t n, uint8_t *d_masks, int64_t masks_len,
                                 ytgb_brick *d_desc, int32_t n_bricks, void *stream) {
    if (n < 0 || masks_len < 0 || (n > 0 && (!src || !count || !dst_offset || !brick || !d_masks || !d_desc))) {
        ytgb_set_error("ytgb_gather_masks: bad arguments");
        return YTGB_ERR_INVALID;
    }
    if (n == 0) return YTGB_OK;
    if (!device_reads_host()) {
        ytgb_set_error("ytgb_gather_masks: the device cannot read pageable host memory");
        return YTGB_ERR_INVALID;
    }
    if ((uintptr_t)d_desc & 7) {
        ytgb_set_error("ytgb_gather_masks: misaligned descriptors");
        return YTGB_ERR_INVALID;
    }
    for (int64_t k = 0; k < n; k++) {
        if (count[k] < 0 || (count[k] > 0 && !src[k]) || dst_offset[k] < 0 || dst_offset[k] > masks_len - count[k] ||
            brick[k] < 0 || brick[k] >= n_bricks) {
            ytgb_set_error("ytgb_gather_masks: mask " + std::to_string(k) + " is null, does not fit the arena or "
                           "names no brick");
            return YTGB_ERR_INVALID;
        }
    }
    const int blocks = (int)(n < 152 * 16 ? n : 152 * 16);
    gather_masks_kernel<<<blocks, GATHER_BLOCK, 0, (cudaStream_t)stream>>>(src, count, dst_offset, brick, n, d_masks,
                                                                          d_desc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("ytgb_gather_masks: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return YTGB_OK;
}

extern "C" int ytgb_vertex_bricks(const double *d_cells, int64_t n_cells, const int64_t *d_grid_offset,
                                  const int32_t *d_grid_dims, int32_t n_grids, const int32_t *d_brick_grid,
                                  const int32_t *d_brick_lo, const ytgb_brick *d_bricks, int32_t n_bricks,
                                  int32_t field, int32_t log_field, float *d_arena, int64_t arena_len,
                                  int32_t *d_error, void *stream, float *d_arena_lo) {
    if (n_bricks < 0 || n_grids < 0 || n_cells < 0 || arena_len < 0 || field < 0 || field > 5) {
        ytgb_set_error("ytgb_vertex_bricks: bad sizes");
        return YTGB_ERR_INVALID;
    }
    if (n_bricks == 0) return YTGB_OK;
    if (!d_cells || !d_grid_offset || !d_grid_dims || !d_brick_grid || !d_brick_lo || !d_bricks || !d_arena ||
        ((uintptr_t)d_cells & 7) || ((uintptr_t)d_grid_offset & 7) || ((uintptr_t)d_grid_dims & 3) ||
        ((uintptr_t)d_brick_grid & 3) || ((uintptr_t)d_brick_lo & 3) || ((uintptr_t)d_bricks & 7) ||
        ((uintptr_t)d_arena & 3) || ((uintptr_t)d_error & 3) || ((uintptr_t)d_arena_lo & 3)) {
        ytgb_set_error("ytgb_vertex_bricks: null or misaligned device array");
        return YTGB_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    vertex_bricks_kernel<<<n_bricks, PREP_BLOCK, 0, s>>>(d_cells, n_cells, d_grid_offset, d_grid_dims, n_grids,
                                                          d_brick_grid, d_brick_lo, d_bricks, field, log_field,
                                                          d_arena, arena_len, d_error, d_arena_lo);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("ytgb_vertex_bricks: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return YTGB_OK;
}
