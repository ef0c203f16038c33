// ytgb_offaxis.cu -- octree off-axis projection by cell splatting.
//
// add_cells_to_image_offaxis (image_utilities.pyx:167-289) projects every
// cell of an octree dataset along the camera's normal: the cell's projected
// square is cut into jmax x kmax sub-squares ("subcells", jmax = kmax =
// 2^depth, capped by the stamp extent), each weighted by the precomputed
// stamp of that depth (the projected thickness of a unit cube) and spread
// bilinearly over the pixels it overlaps (_add_cell_to_image_offaxis,
// :46-165).
//
// The per-subcell weights are separable: subcell (j, k) gives pixel (P, Q)
//     stamp[j][k] * fx_j(P) * fy_k(Q) * dx^3 Nx Ny * q,
// with fx_j(P) = dvx_j where P is the subcell's left pixel jj1 and
// 1 - dvx_j where P is its right pixel jj2 (likewise in y).  The reference
// evaluates the boundaries ((j - jmax/2) dx_loc + x) Nx, their truncations
// and dvx per subcell; here they are evaluated once per row and column of
// subcells, with the same float64 operations in the same order, into a
// per-warp table, so every subcell lands on exactly the reference's pixels
// with the reference's dvx, dvy.  One warp then handles one cell: each lane
// owns one pixel column Q (and a share of the rows j), sums
// stamp[j][k] * fy_k(Q) over the few k that touch Q, spreads the row sum
// over P with fx_j, and adds each finished pixel to the image with one
// float64 atomic per buffer, scaled by dx^3 Nx Ny q (resp. w).  Only the
// association of the products differs from the reference: the sums are
// float64 fused multiply-adds, a few roundings per contribution.  Cells whose rows exceed the table take the
// reference's per-subcell loop (with atomics) instead.
#include <cuda_runtime.h>
#include <cstdint>
#include <string>

#include "ytgb.h"
#include "ytgb_internal.h"
#include "ytgb_ray.cuh"

namespace {

using namespace ytgb;

constexpr int OA_BLOCK = 128;
constexpr int OA_WARPS = OA_BLOCK / 32;
constexpr int OA_KT = 256;  // subcells per row or column held in the table

constexpr int OA_MAXK = 10;  // subcells of a row meeting one pixel column, held in registers

struct AxisTable {
    int edge[OA_KT + 1];  // (int) of the subcell boundaries, in pixels
    double dv[OA_KT];     // fclip((edge[i+1] - b_i) / (b_{i+1} - b_i), 0, 1)
    double uv[OA_KT];     // 1 - dv
};

// fp_utils.pxd:17-40 (fmax, fmin, fclip)
__device__ __forceinline__ double fpmax(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double fpmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double fclip(double f, double a, double b) { return fpmin(fpmax(f, a), b); }

// Subcell boundary i of an axis in pixels: ((i - m / 2.) * d_loc + x) * N
// (image_utilities.pyx:110-111, 124-125)
__device__ __forceinline__ double boundary(int i, int m, double d_loc, double x, int N) {
    return ytgb::dmul(ytgb::dadd(ytgb::dmul(ytgb::dsub((double)i, (double)m * 0.5), d_loc), x), (double)N);
}

// Entry i of an axis table: boundaries i and i + 1, their truncations and
// dv (image_utilities.pyx:110-120 and 124-138); entry m - 1 also stores the
// last edge.
__device__ __forceinline__ void fill_entry(AxisTable &t, int i, int m, double d_loc, double x, int N) {
    const double b0 = boundary(i, m, d_loc, x, N), b1 = boundary(i + 1, m, d_loc, x, N);
    const int e1 = __double2int_rz(b1);
    t.edge[i] = __double2int_rz(b0);
    if (i == m - 1) t.edge[m] = e1;
    const double dv = fclip(ytgb::ddiv(ytgb::dsub((double)e1, b0), ytgb::dsub(b1, b0)), 0.0, 1.0);
    t.dv[i] = dv;
    t.uv[i] = ytgb::dsub(1.0, dv);
}

// ceil(log2(v)) for finite v > 1 as the C library's log2 gives it: E for
// v = 2^E exactly, E + 1 when v lies more than 2^12 ulps above 2^E (log2(v)
// then exceeds E by over ten of its own ulps), and the library log2 in the
// narrow band between.
__device__ __forceinline__ int ceil_log2_above1(double v) {
    const long long b = dbits(v);
    const int E = (int)(b >> 52) - 1023;
    const long long f = b & MANT52;
    if (f == 0) return E;
    if (f >= 4096) return E + 1;
    return __double2int_rz(ceil(log2(v)));
}

// smallest k in [0, m) with edge[k + 1] >= Q (m if none)
__device__ __forceinline__ int first_reaching(const AxisTable &t, int m, int Q) {
    int lo = 0, hi = m;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (t.edge[mid + 1] >= Q) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// largest k in [0, m) with edge[k] <= Q (-1 if none)
__device__ __forceinline__ int last_starting(const AxisTable &t, int m, int Q) {
    int lo = 0, hi = m;  // first k with edge[k] > Q, minus one
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (t.edge[mid] > Q) hi = mid;
        else lo = mid + 1;
    }
    return lo - 1;
}

struct PixelRun {
    int P = -1;
    double acc = 0.0;
};

__device__ __forceinline__ void flush(PixelRun &r, double *buf, double *bufw, long long Q, int nx, long long npix,
                                      double cq, double cw) {
    if (r.P >= 0) {
        const long long idx = (long long)r.P * nx + Q;
        if (idx < npix) {
            atomicAdd(buf + idx, ytgb::dmul(r.acc, cq));
            atomicAdd(bufw + idx, ytgb::dmul(r.acc, cw));
        }
    }
}

// acc += t * f for pixel P, flushing the previous pixel when P moves on
// (the pixels of a column arrive in nondecreasing order)
__device__ __forceinline__ void add_to(PixelRun &r, int P, double t, double f, double *buf, double *bufw, long long Q,
                                       int nx, long long npix, double cq, double cw) {
    if (P != r.P) {
        flush(r, buf, bufw, Q, nx, npix, cq, cw);
        r.P = P;
        r.acc = 0.0;
    }
    r.acc = __fma_rn(t, f, r.acc);
}

struct Column {
    const double *stamp;  // this depth's stamp
    long long nsy;
    int klo, kcap, Q, nx;  // kcap: the last subcell of a row
    long long npix;
    double cq, cw;
    double *buf, *bufw;
};

// One pixel column Q over the subcell rows [j0, j1): the row's sum of
// stamp[j][k] * fy_k(Q) over the N subcells k = klo .. klo + N - 1 that
// meet Q (weights w), spread over the row's two pixels with dvx, 1 - dvx.
template <int N>
__device__ __forceinline__ void column_rows(const AxisTable &tx, const Column &c, const double (&wk)[OA_MAXK], int j0,
                                            int j1) {
    PixelRun run;
    for (int j = j0; j < j1; j++) {
        const int e0 = tx.edge[j], e1 = tx.edge[j + 1];
        if (e1 < 0 || e0 >= c.nx) continue;  // image_utilities.pyx:116
        const double *srow = c.stamp + (long long)j * c.nsy;
        double t = 0.0;
#pragma unroll
        for (int u = 0; u < N; u++) t = __fma_rn(__ldg(srow + min(c.klo + u, c.kcap)), wk[u], t);
        if (e0 >= 0) add_to(run, e0, t, tx.dv[j], c.buf, c.bufw, c.Q, c.nx, c.npix, c.cq, c.cw);
        if (e1 < c.nx) add_to(run, e1, t, tx.uv[j], c.buf, c.bufw, c.Q, c.nx, c.npix, c.cq, c.cw);
    }
    flush(run, c.buf, c.bufw, c.Q, c.nx, c.npix, c.cq, c.cw);
}

// the same with the weights read from the table (more than OA_MAXK subcells
// of a row in one pixel: a very wide image against its height)
__device__ void column_rows_wide(const AxisTable &tx, const AxisTable &ty, const Column &c, int khi, int j0, int j1) {
    PixelRun run;
    for (int j = j0; j < j1; j++) {
        const int e0 = tx.edge[j], e1 = tx.edge[j + 1];
        if (e1 < 0 || e0 >= c.nx) continue;
        const double *srow = c.stamp + (long long)j * c.nsy;
        double t = 0.0;
        for (int k = c.klo; k <= khi; k++) {
            const double st = __ldg(srow + k);
            if (ty.edge[k] == c.Q) t = __fma_rn(st, ty.dv[k], t);
            if (ty.edge[k + 1] == c.Q) t = __fma_rn(st, ty.uv[k], t);
        }
        if (e0 >= 0) add_to(run, e0, t, tx.dv[j], c.buf, c.bufw, c.Q, c.nx, c.npix, c.cq, c.cw);
        if (e1 < c.nx) add_to(run, e1, t, tx.uv[j], c.buf, c.bufw, c.Q, c.nx, c.npix, c.cq, c.cw);
    }
    flush(run, c.buf, c.bufw, c.Q, c.nx, c.npix, c.cq, c.cw);
}

// The reference's own per-subcell loop (image_utilities.pyx:105-165) for a
// cell whose subcell rows do not fit the table: lanes over the subcells.
__device__ void cell_direct(const ytgb_offaxis_args &a, int lane, int depth, int jm, int km, double dx_loc,
                            double dy_loc, double x, double y, double dx3, double w, double q) {
    const int nx = a.nx, ny = a.ny;
    const long long npix = (long long)nx * ny;
    const long long n_sub = (long long)jm * km;
    for (long long s = lane; s < n_sub; s += 32) {
        const int j = (int)(s / km), k = (int)(s % km);
        const double xx1 = boundary(j, jm, dx_loc, x, nx), xx2 = boundary(j + 1, jm, dx_loc, x, nx);
        const int jj1 = __double2int_rz(xx1), jj2 = __double2int_rz(xx2);
        if (jj2 < 0 || jj1 >= nx) continue;
        const double dvx = fclip(ytgb::ddiv(ytgb::dsub((double)jj2, xx1), ytgb::dsub(xx2, xx1)), 0.0, 1.0);
        const double st = __ldg(a.stamp + ((long long)depth * a.nsx + j) * a.nsy + k);
        if (st == 0.0) continue;  // outside the stamp's mask
        const double yy1 = boundary(k, km, dy_loc, y, ny), yy2 = boundary(k + 1, km, dy_loc, y, ny);
        const int kk1 = __double2int_rz(yy1), kk2 = __double2int_rz(yy2);
        if (kk2 < 0 || kk1 >= ny) continue;
        const double tmp = ytgb::dmul(st, dx3);
        const double sw = ytgb::dmul(tmp, w), sq = ytgb::dmul(tmp, q);
        const double dvy = fclip(ytgb::ddiv(ytgb::dsub((double)kk2, yy1), ytgb::dsub(yy2, yy1)), 0.0, 1.0);
        const double ux = ytgb::dsub(1.0, dvx), uy = ytgb::dsub(1.0, dvy);
        long long idx;
        double f;
        if (jj1 >= 0 && kk1 >= 0 && (idx = (long long)jj1 * nx + kk1) < npix) {
            f = ytgb::dmul(dvx, dvy);
            atomicAdd(a.buffer + idx, ytgb::dmul(sq, f));
            atomicAdd(a.buffer_weight + idx, ytgb::dmul(sw, f));
        }
        if (jj1 >= 0 && kk2 < ny && (idx = (long long)jj1 * nx + kk2) < npix) {
            f = ytgb::dmul(dvx, uy);
            atomicAdd(a.buffer + idx, ytgb::dmul(sq, f));
            atomicAdd(a.buffer_weight + idx, ytgb::dmul(sw, f));
        }
        if (jj2 < nx && kk1 >= 0 && (idx = (long long)jj2 * nx + kk1) < npix) {
            f = ytgb::dmul(ux, dvy);
            atomicAdd(a.buffer + idx, ytgb::dmul(sq, f));
            atomicAdd(a.buffer_weight + idx, ytgb::dmul(sw, f));
        }
        if (jj2 < nx && kk2 < ny && (idx = (long long)jj2 * nx + kk2) < npix) {
            f = ytgb::dmul(ux, uy);
            atomicAdd(a.buffer + idx, ytgb::dmul(sq, f));
            atomicAdd(a.buffer_weight + idx, ytgb::dmul(sw, f));
        }
    }
}

__global__ void __launch_bounds__(OA_BLOCK) offaxis_kernel(const ytgb_offaxis_args a, int32_t *error) {
    __shared__ AxisTable s_x[OA_WARPS], s_y[OA_WARPS];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    AxisTable &tx = s_x[wib], &ty = s_y[wib];
    const int nx = a.nx, ny = a.ny;
    const long long npix = (long long)nx * ny;
    const double sq3 = ytgb::dsqrt(3.0);
    const double sq3x4 = ytgb::dmul(4.0, sq3);
    const double nmax = nx > ny ? (double)nx : (double)ny;  // fmax(Nx, Ny)
    const long long n_warps = (long long)gridDim.x * OA_WARPS;
    for (long long c = (long long)blockIdx.x * OA_WARPS + wib; c < a.n; c += n_warps) {
        const double dx = __ldg(a.dxp + c), w = __ldg(a.weight + c), q = __ldg(a.qty + c);
        const double X0 = __ldg(a.xp + 3 * c), X1 = __ldg(a.xp + 3 * c + 1), X2 = __ldg(a.xp + 3 * c + 2);
        if (!(dx > 0.0) || !isfinite(dx)) {
            if (lane == 0 && error) atomicCAS(error, 0, YTGB_DEVERR_BAD_CELL);
            continue;
        }
        // image_utilities.pyx:264-276 and :66-80
        const double cmw = ytgb::dmul(dx, sq3);
        const double x = ytgb::dadd(ytgb::dadd(ytgb::dadd(ytgb::dmul(a.rot[0], X0), ytgb::dmul(a.rot[1], X1)), ytgb::dmul(a.rot[2], X2)), 0.5);
        const double y = ytgb::dadd(ytgb::dadd(ytgb::dadd(ytgb::dmul(a.rot[3], X0), ytgb::dmul(a.rot[4], X1)), ytgb::dmul(a.rot[5], X2)), 0.5);
        const double half = ytgb::dmul(cmw, 0.5);  // cmw / 2, exactly
        const double dx3 = ytgb::dmul(ytgb::dmul(ytgb::dmul(ytgb::dmul(dx, dx), dx), (double)nx), (double)ny);
        const double lx = ytgb::dsub(x, half), rx = ytgb::dadd(x, half), ly = ytgb::dsub(y, half), ry = ytgb::dadd(y, half);
        const int jmin = max(__double2int_rz(floor(ytgb::dmul(lx, (double)nx))), 0);
        const int jmax = max(__double2int_rz(ceil(ytgb::dmul(rx, (double)nx))), nx - 1);
        const int kmin = min(__double2int_rz(floor(ytgb::dmul(ly, (double)ny))), 0);
        const int kmax = max(__double2int_rz(ceil(ytgb::dmul(ry, (double)ny))), ny - 1);
        if (jmax == jmin + 1 && kmax == kmin + 1) {  // :83-87, the cell inside one pixel
            const long long idx = (long long)jmin * nx + kmin;
            if (lane == 0 && idx >= 0 && idx < npix) {
                atomicAdd(a.buffer + idx, ytgb::dmul(q, dx3));
                atomicAdd(a.buffer_weight + idx, ytgb::dmul(w, dx3));
            }
            continue;
        }
        // :92-99: the stamp level with at least 4 subcells per pixel diagonal
        const double v = ytgb::dmul(ytgb::dmul(sq3x4, dx), nmax);
        int depth = v > 1.0 ? ceil_log2_above1(v) : 1;
        depth = depth < 1 ? 1 : (depth > a.max_depth - 1 ? a.max_depth - 1 : depth);
        const int jm = min(a.nsx, 1 << depth), km = min(a.nsy, 1 << depth);
        // cmw / 2^depth is an exact scaling
        const double pw = dfrom((long long)(1023 - depth) << 52);
        const double dx_loc = jm == (1 << depth) ? ytgb::dmul(cmw, pw) : ytgb::ddiv(cmw, (double)jm);
        const double dy_loc = km == (1 << depth) ? ytgb::dmul(cmw, pw) : ytgb::ddiv(cmw, (double)km);
        const double cq = ytgb::dmul(dx3, q), cw = ytgb::dmul(dx3, w);
        if (jm > OA_KT || km > OA_KT) {
            cell_direct(a, lane, depth, jm, km, dx_loc, dy_loc, x, y, dx3, w, q);
            continue;
        }
        __syncwarp();
        for (int e = lane; e < jm + km; e += 32) {
            if (e < jm) fill_entry(tx, e, jm, dx_loc, x, nx);
            else fill_entry(ty, e - jm, km, dy_loc, y, ny);
        }
        __syncwarp();
        // pixels the cell can reach (the edges are nondecreasing)
        const int Plo = max(tx.edge[0], 0), Phi = min(tx.edge[jm], nx - 1);
        const int Qlo = max(ty.edge[0], 0), Qhi = min(ty.edge[km], ny - 1);
        if (Plo > Phi || Qlo > Qhi) continue;
        // lanes: pixel columns Q (wp of them), times groups sharing out the rows
        const int wy = Qhi - Qlo + 1;
        const int wp = wy < 32 ? wy : 32;
        const int groups = 32 / wp;
        const int g = lane / wp;
        const int j0 = g * jm / groups, j1 = (g + 1) * jm / groups;
        Column col;
        col.stamp = a.stamp + (long long)depth * a.nsx * a.nsy;
        col.nsy = a.nsy;
        col.kcap = km - 1;
        col.nx = nx;
        col.npix = npix;
        col.cq = cq;
        col.cw = cw;
        col.buf = a.buffer;
        col.bufw = a.buffer_weight;
        const int passes = (wy + wp - 1) / wp;
        for (int pass = 0; pass < passes; pass++) {
            const int Q = Qlo + pass * wp + lane - g * wp;
            const bool act = g < groups && Q <= Qhi;
            int klo = 0, nk = 0;
            if (act) {
                klo = first_reaching(ty, km, Q);
                nk = last_starting(ty, km, Q) - klo + 1;
            }
            col.klo = klo;
            col.Q = Q;
            // one unrolled length for the whole warp: lanes of different
            // lengths would otherwise run their loops one after another
            const int N = __reduce_max_sync(0xffffffffu, nk > 0 ? nk : 0);
            if (!act || nk < 1) continue;
            if (N > OA_MAXK) {
                column_rows_wide(tx, ty, col, klo + nk - 1, j0, j1);
                continue;
            }
            // fy_k(Q) of the subcells meeting Q (image_utilities.pyx:141-159),
            // 0 past this lane's own nk
            double w[OA_MAXK];
#pragma unroll
            for (int u = 0; u < OA_MAXK; u++) {
                const int k = klo + u;
                double wv = 0.0;
                if (u < nk) {
                    if (ty.edge[k] == Q) wv = ty.dv[k];
                    if (ty.edge[k + 1] == Q) wv = ytgb::dadd(wv, ty.uv[k]);
                }
                w[u] = wv;
            }
            switch (N) {
            case 1: column_rows<1>(tx, col, w, j0, j1); break;
            case 2: column_rows<2>(tx, col, w, j0, j1); break;
            case 3: column_rows<3>(tx, col, w, j0, j1); break;
            case 4: column_rows<4>(tx, col, w, j0, j1); break;
            case 5: column_rows<5>(tx, col, w, j0, j1); break;
            case 6: column_rows<6>(tx, col, w, j0, j1); break;
            case 7: column_rows<7>(tx, col, w, j0, j1); break;
            case 8: column_rows<8>(tx, col, w, j0, j1); break;
            case 9: column_rows<9>(tx, col, w, j0, j1); break;
            default: column_rows<10>(tx, col, w, j0, j1); break;
            }
        }
    }
}

}  // namespace

extern "C" int ytgb_offaxis_cells(const ytgb_offaxis_args *args, int32_t *d_error, void *stream) {
    if (!args) {
        ytgb_set_error("ytgb_offaxis_cells: null args");
        return YTGB_ERR_INVALID;
    }
    const ytgb_offaxis_args &a = *args;
    if (a.n < 0 || a.nx < 1 || a.ny < 1 || a.nx > a.ny || a.nsx < 1 || a.nsy < 1 || a.max_depth < 2 ||
        a.max_depth > 30) {
        ytgb_set_error("ytgb_offaxis_cells: bad sizes (nx must not exceed ny; 2 <= max_depth <= 30)");
        return YTGB_ERR_INVALID;
    }
    if (a.n == 0) return YTGB_OK;
    if (!a.xp || !a.dxp || !a.qty || !a.weight || !a.stamp || !a.buffer || !a.buffer_weight ||
        ((uintptr_t)a.xp & 7) || ((uintptr_t)a.dxp & 7) || ((uintptr_t)a.qty & 7) || ((uintptr_t)a.weight & 7) ||
        ((uintptr_t)a.stamp & 7) || ((uintptr_t)a.buffer & 7) || ((uintptr_t)a.buffer_weight & 7) ||
        ((uintptr_t)d_error & 3)) {
        ytgb_set_error("ytgb_offaxis_cells: null or misaligned device array");
        return YTGB_ERR_INVALID;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (a.n + OA_WARPS - 1) / OA_WARPS;
    const long long cap = (long long)(sms > 0 ? sms : 152) * 8;
    const int blocks = (int)(want < cap ? want : cap);
    offaxis_kernel<<<blocks, OA_BLOCK, 0, (cudaStream_t)stream>>>(a, d_error);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ytgb_set_error(std::string("ytgb_offaxis_cells: ") + cudaGetErrorString(e));
        return YTGB_ERR_CUDA;
    }
    return YTGB_OK;
}
