// ytgb_pack.cpp -- host-side marshalling of yt's bricks for one render.
//
// yt's sampler reads each PartitionedGrid's float64 arrays in place, one brick
// per call (image_samplers.pyx:146-197).  The device path wants every brick's
// fields in one float32 arena, so the drop-in sampler gathers them once per
// render.  A single Python/numpy thread does that at a few GB/s; here the
// gather is split over the host's cores.  The float64 -> float32 conversion
// is the C++ cast (round to nearest even), the same rounding as numpy's
// astype(float32).
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "ytgb.h"
#include "ytgb_internal.h"

namespace {

// Default: up to 8 threads.  These loops are memory-bound; on the 16-core
// Grace host a 32 MiB copy ran in 0.46 ms on 4-8 threads and 0.85 ms on 16.
int thread_count(int32_t requested, int64_t work_bytes) {
    int t = requested > 0 ? requested : std::min(8, (int)std::thread::hardware_concurrency());
    if (t < 1) t = 1;
    if (t > 64) t = 64;
    // at least ~1 MiB per thread: below that, thread start-up dominates
    const int64_t by_size = std::max<int64_t>(1, work_bytes >> 20);
    return (int)std::min<int64_t>(t, by_size);
}

// Run body(lo, hi) over [0, total) split into `threads` contiguous ranges.
template <typename F>
void parallel_ranges(int64_t total, int threads, F body) {
    if (threads <= 1 || total <= 0) {
        body((int64_t)0, total);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(threads - 1);
    const int64_t step = (total + threads - 1) / threads;
    for (int t = 1; t < threads; t++) {
        const int64_t lo = std::min(total, t * step), hi = std::min(total, (t + 1) * step);
        pool.emplace_back([=] { body(lo, hi); });
    }
    body(0, std::min(total, step));
    for (auto &th : pool) th.join();
}

// Elements [lo, hi) of the concatenation of n arrays with prefix sums `start`
// (start[k] = first element of array k, start[n] = total): calls
// f(k, first, last) for each piece of array k inside the range.
template <typename F>
void for_pieces(const std::vector<int64_t> &start, int64_t lo, int64_t hi, F f) {
    if (lo >= hi) return;
    int64_t k = std::upper_bound(start.begin(), start.end(), lo) - start.begin() - 1;
    const int64_t n = (int64_t)start.size() - 1;
    for (; k < n && start[k] < hi; k++) {
        const int64_t a = std::max(lo, start[k]) - start[k];
        const int64_t b = std::min(hi, start[k + 1]) - start[k];
        if (b > a) f(k, a, b);
    }
}

template <typename T>
int check_lists(const T *const *src, const int64_t *count, const int64_t *dst_offset, int64_t n, const void *dst,
                std::vector<int64_t> &start, const char *who) {
    if (n < 0 || (n > 0 && (!src || !count || !dst_offset || !dst))) {
        ytgb_set_error(std::string(who) + ": null argument");
        return YTGB_ERR_INVALID;
    }
    start.assign(n + 1, 0);
    for (int64_t k = 0; k < n; k++) {
        if (count[k] < 0 || dst_offset[k] < 0 || (count[k] > 0 && !src[k])) {
            ytgb_set_error(std::string(who) + ": bad array " + std::to_string(k));
            return YTGB_ERR_INVALID;
        }
        start[k + 1] = start[k] + count[k];
    }
    return YTGB_OK;
}

}  // namespace

extern "C" int ytgb_pack_fields(const double *const *src, const int64_t *count, const int64_t *dst_offset,
                                int64_t n, float *dst, int32_t n_threads) {
    std::vector<int64_t> start;
    if (int st = check_lists(src, count, dst_offset, n, dst, start, "ytgb_pack_fields")) return st;
    const int64_t total = start[n];
    parallel_ranges(total, thread_count(n_threads, total * 12), [&](int64_t lo, int64_t hi) {
        for_pieces(start, lo, hi, [&](int64_t k, int64_t a, int64_t b) {
            const double *s = src[k];
            float *d = dst + dst_offset[k];
            for (int64_t i = a; i < b; i++) d[i] = (float)s[i];
        });
    });
    return YTGB_OK;
}

extern "C" int ytgb_pack_fields_split(const double *const *src, const int64_t *count, const int64_t *dst_offset,
                                      int64_t n, float *dst_hi, float *dst_lo, int32_t n_threads) {
    std::vector<int64_t> start;
    if (int st = check_lists(src, count, dst_offset, n, dst_hi, start, "ytgb_pack_fields_split")) return st;
    if (n > 0 && !dst_lo) {
        ytgb_set_error("ytgb_pack_fields_split: null low-part arena");
        return YTGB_ERR_INVALID;
    }
    const int64_t total = start[n];
    parallel_ranges(total, thread_count(n_threads, total * 16), [&](int64_t lo, int64_t hi) {
        for_pieces(start, lo, hi, [&](int64_t k, int64_t a, int64_t b) {
            const double *s = src[k];
            float *dh = dst_hi + dst_offset[k];
            float *dl = dst_lo + dst_offset[k];
            for (int64_t i = a; i < b; i++) {
                const float h = (float)s[i];
                dh[i] = h;
                // the float32 rounding error, itself rounded to float32
                // (NaN and infinities carry 0)
                const double r = s[i] - (double)h;
                dl[i] = r == r && r - r == 0.0 ? (float)r : 0.0f;
            }
        });
    });
    return YTGB_OK;
}

extern "C" int ytgb_pack_masks(const uint8_t *const *src, const int64_t *count, const int64_t *dst_offset,
                               int64_t n, uint8_t *dst, int32_t n_threads, int32_t *all_ones) {
    std::vector<int64_t> start;
    if (int st = check_lists(src, count, dst_offset, n, dst ? (const void *)dst : (const void *)all_ones, start,
                             "ytgb_pack_masks"))
        return st;
    if (!all_ones) {
        ytgb_set_error("ytgb_pack_masks: null all_ones");
        return YTGB_ERR_INVALID;
    }
    const int64_t total = start[n];
    const int threads = thread_count(n_threads, total * 2);
    std::vector<int> ones(threads > 0 ? threads : 1, 1);
    const int64_t step = threads > 1 ? (total + threads - 1) / threads : total;
    parallel_ranges(total, threads, [&](int64_t lo, int64_t hi) {
        const int slot = step > 0 ? (int)(lo / step) : 0;
        int ok = 1;
        for_pieces(start, lo, hi, [&](int64_t k, int64_t a, int64_t b) {
            const uint8_t *s = src[k];
            if (dst) std::memcpy(dst + dst_offset[k] + a, s + a, (size_t)(b - a));
            for (int64_t i = a; i < b && ok; i++) ok = s[i] == 1;
        });
        ones[slot] = ok;
    });
    *all_ones = 1;
    for (int v : ones) *all_ones &= v;
    return YTGB_OK;
}

extern "C" int ytgb_host_is_uniform(const double *x, int64_t n, double value, int32_t n_threads, int32_t *result) {
    if (n < 0 || (n > 0 && !x) || !result) {
        ytgb_set_error("ytgb_host_is_uniform: bad arguments");
        return YTGB_ERR_INVALID;
    }
    uint64_t want;
    std::memcpy(&want, &value, sizeof(want));
    const int threads = thread_count(n_threads, n * 8);
    std::vector<int> same(threads > 0 ? threads : 1, 1);
    const int64_t step = threads > 1 ? (n + threads - 1) / threads : n;
    parallel_ranges(n, threads, [&](int64_t lo, int64_t hi) {
        const int slot = step > 0 ? (int)(lo / step) : 0;
        int ok = 1;
        for (int64_t i = lo; i < hi && ok; i++) {
            uint64_t b;
            std::memcpy(&b, x + i, sizeof(b));
            ok = b == want;
        }
        same[slot] = ok;
    });
    *result = 1;
    for (int v : same) *result &= v;
    return YTGB_OK;
}

extern "C" int ytgb_host_copy(void *dst, const void *src, int64_t bytes, int32_t n_threads) {
    if (bytes < 0 || (bytes > 0 && (!dst || !src))) {
        ytgb_set_error("ytgb_host_copy: bad arguments");
        return YTGB_ERR_INVALID;
    }
    unsigned char *d = static_cast<unsigned char *>(dst);
    const unsigned char *s = static_cast<const unsigned char *>(src);
    parallel_ranges(bytes, thread_count(n_threads, bytes * 2), [&](int64_t lo, int64_t hi) {
        if (hi > lo) std::memcpy(d + lo, s + lo, (size_t)(hi - lo));
    });
    return YTGB_OK;
}

// MADV_POPULATE_WRITE (Linux 5.14) where the C library headers predate it.
#ifndef MADV_POPULATE_WRITE
#define MADV_POPULATE_WRITE 23
#endif

extern "C" int ytgb_host_prefault(void *p, int64_t bytes) {
    if (bytes < 0 || (bytes > 0 && !p)) {
        ytgb_set_error("ytgb_host_prefault: bad arguments");
        return YTGB_ERR_INVALID;
    }
    const long page = sysconf(_SC_PAGESIZE);
    if (page <= 0 || bytes == 0) return YTGB_OK;
    const uintptr_t a = (uintptr_t)p, e = a + (uintptr_t)bytes;
    const uintptr_t lo = (a + page - 1) / page * page, hi = e / page * page;
    if (hi <= lo) return YTGB_OK;
    // whole pages inside [p, p + bytes) only, split over host threads (the
    // kernel zero-fills each new page: one thread populated a 32 MiB image
    // in ~1 ms on the Grace host); failure (older kernel, an unusual
    // mapping) just leaves the pages to fault on first write
    const int64_t pages = (int64_t)((hi - lo) / page);
    parallel_ranges(pages, thread_count(0, (int64_t)(hi - lo)), [&](int64_t p0, int64_t p1) {
        if (p1 > p0) (void)madvise((void *)(lo + p0 * page), (size_t)((p1 - p0) * page), MADV_POPULATE_WRITE);
    });
    return YTGB_OK;
}
