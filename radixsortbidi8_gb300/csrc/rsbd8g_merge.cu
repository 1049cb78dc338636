// rsbd8g_merge.cu - stable merges of sorted runs (rsbd8g_merge_runs) and the chunked sort of host
// arrays larger than the device can hold (rsbd8g_radixsortcopy_chunked), built on them.
//
//   rsbd8g_merge_runs            k sorted runs back to back in device memory -> one sorted array:
//                                rounds of pairwise merges (k_merge2), ping-ponging between the
//                                caller's buffer and the output so the last round lands in output
//   rsbd8g_radixsortcopy_chunked a host array sorted in chunks that fit the given device budget
//                                (each chunk: copy in, radix sort in place, copy back into a host
//                                run buffer), then merged block by block: the host finds where
//                                each output block starts in every run (a search on the host
//                                copies), the runs' spans of the block are copied to the device,
//                                merged there and copied back into the output.
// The reference merges the halves or thirds that its threads sorted (mergehalves* / mergethirds*,
// Radixsortbidi8.hpp:54437-56418, dispatched at :55150-55160 and :56560-56569); the same merge
// order -- filtered key, then run precedence on ties -- takes the parts of an array that does not
// fit the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "rsbd8g.h"
#include "rsbd8g_internal.h"
#include "rsbd8g_merge.cuh"

namespace rsbd8g {
namespace {

constexpr int kMergeThreads = 256;
// outputs per thread and tile: 4096-key tiles up to 4-byte keys; 2048 for 8-byte keys (four CTAs of
// 49 KB per SM instead of two of 97 KB: 2^28 int64 merge 1.51 -> 1.34 ms; 4-byte keys were slower
// with 2048-key tiles, 0.82 -> 0.93 ms) and 1024 for 16-byte keys
template <typename U>
constexpr int merge_items() { return sizeof(U) >= 16 ? 4 : (sizeof(U) == 8 ? 8 : 16); }

template <typename U, int MODE>
cudaError_t launch_merge2_t(const U *A, uint64_t na, const U *B, uint64_t nb, U *out, bool desc, bool a_first,
                            cudaStream_t s) {
    constexpr int IT = merge_items<U>();
    using L = MergeSmem<U, kMergeThreads, IT>;
    auto kern = k_merge2<U, MODE, kMergeThreads, IT>;
    int dev = 0;
    cudaGetDevice(&dev);
    static std::once_flag once[64];
    static int occ[64];
    std::call_once(once[dev & 63], [&] {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(L::kBytes));
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, kMergeThreads, L::kBytes);
        occ[dev & 63] = b > 0 ? b : 1;
    });
    const uint64_t total = na + nb;
    if (total == 0) return cudaSuccess;
    // persistent CTAs, each a contiguous range of whole tiles of the output
    const uint64_t tiles = (total + L::kTile - 1) / L::kTile;
    const uint64_t resident = uint64_t(occ[dev & 63]) * device_sms(dev);
    const uint64_t per = (tiles + resident - 1) / resident * L::kTile;
    const uint64_t grid = (total + per - 1) / per;
    LaunchTimer t(s, RSBD8G_KERNEL_MERGE, uint32_t(sizeof(U)), 0, total);
    kern<<<uint32_t(grid), kMergeThreads, L::kBytes, s>>>(A, na, B, nb, out, desc ? 1u : 0u, a_first ? 1u : 0u, per);
    return cudaGetLastError();
}

template <typename U>
cudaError_t launch_merge2(const Resolved &r, const void *A, uint64_t na, const void *B, uint64_t nb, void *out,
                          cudaStream_t s) {
    const int mode = int(r.f.absv | (r.f.sign << 1) | (r.f.fltp << 2));
    const bool desc = r.f.desc != 0, a_first = r.rev == 0;   // the earlier run wins ties in forward order
    cudaError_t e;
#define RSBD8G_MERGE(M)                                                                                     \
    e = launch_merge2_t<U, M>(static_cast<const U *>(A), na, static_cast<const U *>(B), nb, static_cast<U *>(out), \
                              desc, a_first, s)
    RSBD8G_MODE_SWITCH(mode, RSBD8G_MERGE)
#undef RSBD8G_MERGE
    return e;
}

cudaError_t merge2(const Resolved &r, const void *A, uint64_t na, const void *B, uint64_t nb, void *out,
                   cudaStream_t s) {
    switch (r.key_bytes) {
        case 1: return launch_merge2<uint8_t>(r, A, na, B, nb, out, s);
        case 2: return launch_merge2<uint16_t>(r, A, na, B, nb, out, s);
        case 4: return launch_merge2<uint32_t>(r, A, na, B, nb, out, s);
        case 8: return launch_merge2<uint64_t>(r, A, na, B, nb, out, s);
        default:
            return r.x87 ? launch_merge2<KeyX87>(r, A, na, B, nb, out, s)
                         : launch_merge2<KeyU128>(r, A, na, B, nb, out, s);
    }
}

// Rounds of pairwise merges of the runs lying back to back in `in` (lengths `len`, in run order):
// runs 2i and 2i + 1 merge into one, an odd last run is copied.  Round 1 reads `in` and writes
// `x`, round 2 reads `x` and writes `y`, round 3 writes `x` again, and so on (`y` may be `in`: it
// is not read after round 1).  *result is where the merged array ends up (`in` for a single run).
cudaError_t merge_rounds(const Resolved &r, std::vector<uint64_t> len, const void *in, void *x, void *y,
                         cudaStream_t s, const void **result) {
    const size_t es = r.elem_bytes;
    const unsigned char *src = static_cast<const unsigned char *>(in);
    for (int round = 0; len.size() > 1; ++round) {
        unsigned char *dst = static_cast<unsigned char *>(round % 2 == 0 ? x : y);
        std::vector<uint64_t> next;
        uint64_t off = 0;
        for (size_t i = 0; i < len.size(); i += 2) {
            cudaError_t e;
            if (i + 1 < len.size()) {
                e = merge2(r, src + off * es, len[i], src + (off + len[i]) * es, len[i + 1], dst + off * es, s);
                next.push_back(len[i] + len[i + 1]);
            } else {
                e = len[i] ? cudaMemcpyAsync(dst + off * es, src + off * es, len[i] * es, cudaMemcpyDeviceToDevice, s)
                           : cudaSuccess;
                next.push_back(len[i]);
            }
            if (e != cudaSuccess) return e;
            off += next.back();
        }
        len.swap(next);
        src = dst;
    }
    *result = src;
    return cudaSuccess;
}

// rounds of merging needed for k runs
int merge_round_count(size_t k) {
    int rounds = 0;
    for (; k > 1; k = (k + 1) / 2) ++rounds;
    return rounds;
}

// ---- host-side search of the merge order (the chunked sort's block boundaries) -----------------

template <typename U, int MODE>
struct HostRuns {
    std::vector<const U *> run;
    std::vector<uint64_t> len;
    bool desc, rev;

    // precedence on equal keys: the earlier run in forward order, the later one under isrevorder
    bool prec(size_t r, size_t s) const { return rev ? r > s : r < s; }
    // elements of run s that go before element x of run r
    uint64_t before(size_t s, size_t r, U x) const {
        const U kx = order_key<MODE>(x, desc);
        const bool ties_before = prec(s, r);
        uint64_t lo = 0, hi = len[s];
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            const U km = order_key<MODE>(run[s][mid], desc);
            const bool b = ties_before ? !key_less(kx, km) : key_less(km, kx);
            if (b) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    }
    // position of element i of run r in the merged order
    uint64_t rank(size_t r, uint64_t i) const {
        uint64_t p = i;
        for (size_t s = 0; s < run.size(); ++s)
            if (s != r) p += before(s, r, run[r][i]);
        return p;
    }
    // elements of every run among the first o of the merged order
    void split(uint64_t o, std::vector<uint64_t> &at) const {
        at.assign(run.size(), 0);
        for (size_t r = 0; r < run.size(); ++r) {
            uint64_t lo = 0, hi = len[r];        // the ranks of a run's elements increase with the index
            while (lo < hi) {
                const uint64_t mid = (lo + hi) >> 1;
                if (rank(r, mid) < o) lo = mid + 1;
                else hi = mid;
            }
            at[r] = lo;
        }
    }
};

template <typename U, int MODE>
void host_split_t(const Resolved &r, const unsigned char *runs, const std::vector<uint64_t> &len, uint64_t o,
                  std::vector<uint64_t> &at) {
    HostRuns<U, MODE> h;
    uint64_t off = 0;
    for (uint64_t l : len) {
        h.run.push_back(reinterpret_cast<const U *>(runs) + off);
        h.len.push_back(l);
        off += l;
    }
    h.desc = r.f.desc != 0;
    h.rev = r.rev != 0;
    h.split(o, at);
}

template <typename U>
void host_split_u(const Resolved &r, const unsigned char *runs, const std::vector<uint64_t> &len, uint64_t o,
                  std::vector<uint64_t> &at) {
    const int mode = int(r.f.absv | (r.f.sign << 1) | (r.f.fltp << 2));
#define RSBD8G_SPLIT(M) host_split_t<U, M>(r, runs, len, o, at)
    RSBD8G_MODE_SWITCH(mode, RSBD8G_SPLIT)
#undef RSBD8G_SPLIT
}

void host_split(const Resolved &r, const unsigned char *runs, const std::vector<uint64_t> &len, uint64_t o,
                std::vector<uint64_t> &at) {
    switch (r.key_bytes) {
        case 1: host_split_u<uint8_t>(r, runs, len, o, at); break;
        case 2: host_split_u<uint16_t>(r, runs, len, o, at); break;
        case 4: host_split_u<uint32_t>(r, runs, len, o, at); break;
        case 8: host_split_u<uint64_t>(r, runs, len, o, at); break;
        default:
            if (r.x87) host_split_u<KeyX87>(r, runs, len, o, at);
            else host_split_u<KeyU128>(r, runs, len, o, at);
            break;
    }
}

// device memory of the in-place sorts of an n-element array cut into chunks of c: a chunk, its
// ping-pong buffer, and the larger scratch of a full chunk and the last one (the tile size, and
// with it the scratch, depends on the count)
size_t chunk_bytes(const Resolved &r, uint64_t n, uint64_t c) {
    const size_t a = (size_t(c) * r.elem_bytes + 255) & ~size_t(255);
    const uint64_t last = n - (n - 1) / c * c;
    return 2 * a + std::max(layout_for(r, c).total, layout_for(r, last).total);
}

struct DeviceAlloc {
    void *p = nullptr;
    ~DeviceAlloc() {
        if (p) cudaFree(p);
    }
};
struct HostAlloc {
    void *p = nullptr;
    bool pinned = false;
    ~HostAlloc() {
        if (!p) return;
        if (pinned) cudaFreeHost(p);
        else std::free(p);
    }
};

}  // namespace

rsbd8g_status chunked_sort(const Resolved &r, uint64_t n, const void *input, void *output, size_t budget,
                           cudaStream_t s) {
    const size_t es = r.elem_bytes;
    // the largest chunk whose in-place sort fits the budget
    uint64_t c = std::min<uint64_t>(n, std::max<uint64_t>(2, budget / (2 * es)));
    while (c > 2 && chunk_bytes(r, n, c) > budget) c -= std::max<uint64_t>(1, c / 64);
    if (chunk_bytes(r, n, c) > budget || c < 2) return RSBD8G_ERR_TOO_LARGE;
    const uint64_t nchunks = (n + c - 1) / c;
    std::vector<uint64_t> len;
    for (uint64_t i = 0; i < nchunks; ++i) len.push_back(std::min<uint64_t>(c, n - i * c));
    DeviceAlloc dmem;
    const size_t dbytes = chunk_bytes(r, n, c);
    if (cudaMalloc(&dmem.p, dbytes) != cudaSuccess) {
        cudaGetLastError();
        return RSBD8G_ERR_NO_MEMORY;
    }
    unsigned char *d = static_cast<unsigned char *>(dmem.p);
    const size_t abytes = (size_t(c) * es + 255) & ~size_t(255);
    unsigned char *da = d, *db = d + abytes, *dscr = d + 2 * abytes;   // chunk, ping-pong buffer, scratch
    const size_t scr_bytes = dbytes - 2 * abytes;
    // one chunk: the sorted chunk goes straight to the output
    HostAlloc runs_mem;
    unsigned char *runs = static_cast<unsigned char *>(output);
    if (nchunks > 1) {
        if (cudaMallocHost(&runs_mem.p, size_t(n) * es) == cudaSuccess) {
            runs_mem.pinned = true;
        } else {
            cudaGetLastError();
            runs_mem.p = std::malloc(size_t(n) * es);
            if (!runs_mem.p) return RSBD8G_ERR_NO_MEMORY;
        }
        runs = static_cast<unsigned char *>(runs_mem.p);
    }
    // every error return first waits for the copies in flight (they may read or write the buffers
    // freed on return)
    auto fail = [s](rsbd8g_status st) {
        cudaStreamSynchronize(s);
        cudaGetLastError();
        return st;
    };
    // phase 1: each chunk sorted on the device, back into the run buffer
    uint64_t off = 0;
    for (uint64_t i = 0; i < nchunks; ++i) {
        const uint64_t m = len[i];
        if (cudaMemcpyAsync(da, static_cast<const unsigned char *>(input) + off * es, m * es, cudaMemcpyDefault, s) !=
            cudaSuccess)
            return fail(RSBD8G_ERR_CUDA);
        if (m > 1) {
            const rsbd8g_status st = enqueue_sort(r, m, dscr, scr_bytes, da, nullptr, db, true, false, s);
            if (st != RSBD8G_OK) return fail(st);
            const rsbd8g_status dst = read_device_status(dscr, s, false);
            if (dst != RSBD8G_OK) return fail(dst);
        }
        if (cudaMemcpyAsync(runs + off * es, da, m * es, cudaMemcpyDefault, s) != cudaSuccess)
            return fail(RSBD8G_ERR_CUDA);
        off += m;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return fail(RSBD8G_ERR_CUDA);
    if (nchunks == 1) return RSBD8G_OK;
    // phase 2: the merged order block by block; a block's spans and its merge ping-pong fit the
    // chunk allocation (two chunk arrays)
    const uint64_t block = c;
    std::vector<uint64_t> at0(nchunks, 0), at1;
    std::vector<uint64_t> run_off(nchunks, 0);
    for (uint64_t i = 1; i < nchunks; ++i) run_off[i] = run_off[i - 1] + len[i - 1];
    for (uint64_t o = 0; o < n; o += block) {
        const uint64_t o1 = std::min<uint64_t>(n, o + block);
        host_split(r, runs, len, o1, at1);
        std::vector<uint64_t> span;
        uint64_t pos = 0;
        for (uint64_t i = 0; i < nchunks; ++i) {
            const uint64_t m = at1[i] - at0[i];
            span.push_back(m);
            if (m && cudaMemcpyAsync(da + pos * es, runs + (run_off[i] + at0[i]) * es, m * es, cudaMemcpyDefault,
                                     s) != cudaSuccess)
                return fail(RSBD8G_ERR_CUDA);
            pos += m;
        }
        if (pos != o1 - o) return fail(RSBD8G_ERR_DEVICE_FAULT);   // the split is inconsistent: never expected
        // merge the spans: they ping-pong between db and da (da is free once round 1 has read it)
        const void *merged = nullptr;
        if (merge_rounds(r, span, da, db, da, s, &merged) != cudaSuccess) return fail(RSBD8G_ERR_CUDA);
        if (cudaMemcpyAsync(static_cast<unsigned char *>(output) + o * es, merged, pos * es, cudaMemcpyDefault,
                            s) != cudaSuccess)
            return fail(RSBD8G_ERR_CUDA);
        if (cudaStreamSynchronize(s) != cudaSuccess) return fail(RSBD8G_ERR_CUDA);
        at0 = at1;
    }
    return RSBD8G_OK;
}

}  // namespace rsbd8g

// ---- the C ABI ----------------------------------------------------------------------------------

using namespace rsbd8g;

extern "C" {

RSBD8G_API rsbd8g_status rsbd8g_merge_runs(const rsbd8g_desc *desc, size_t nruns, const size_t *run_counts,
                                           const void *input, void *output, void *buffer, rsbd8g_stream stream) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (r.indirect != RSBD8G_DIRECT) return RSBD8G_ERR_BAD_ARG;
    if (nruns == 0) return RSBD8G_OK;
    if (!run_counts) return RSBD8G_ERR_BAD_ARG;
    std::vector<uint64_t> len(run_counts, run_counts + nruns);
    uint64_t total = 0;
    for (uint64_t l : len) {
        if (l > (uint64_t(1) << 40) || total + l > (uint64_t(1) << 40)) return RSBD8G_ERR_TOO_LARGE;
        total += l;
    }
    if (total == 0) return RSBD8G_OK;
    if (!input || !output || input == output) return RSBD8G_ERR_BAD_ARG;
    const int rounds = merge_round_count(nruns);
    if (rounds >= 2 && (!buffer || buffer == input || buffer == output)) return RSBD8G_ERR_BAD_ARG;
    if (r.key_bytes == 16) {
        auto mis = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) != 0; };
        if (mis(input) || mis(output) || (buffer && mis(buffer))) return RSBD8G_ERR_BAD_ARG;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // the rounds alternate between output and buffer so that the last one writes the output
    void *x = (rounds % 2 == 1) ? output : buffer, *y = (rounds % 2 == 1) ? buffer : output;
    const void *result = nullptr;
    if (merge_rounds(r, len, input, x, y, s, &result) != cudaSuccess) return RSBD8G_ERR_CUDA;
    if (result != output &&
        cudaMemcpyAsync(output, result, size_t(total) * r.elem_bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return RSBD8G_ERR_CUDA;
    return RSBD8G_OK;
}

RSBD8G_API rsbd8g_status rsbd8g_radixsortcopy_chunked(const rsbd8g_desc *desc, size_t count, const void *input,
                                                      void *output, size_t device_bytes, rsbd8g_stream stream) {
    Resolved r;
    rsbd8g_status st = resolve(desc, &r);
    if (st != RSBD8G_OK) return st;
    if (r.indirect != RSBD8G_DIRECT) return RSBD8G_ERR_BAD_ARG;
    if (count == 0) return RSBD8G_OK;
    if (!input || !output || input == output) return RSBD8G_ERR_BAD_ARG;
    if (count > (uint64_t(1) << 40)) return RSBD8G_ERR_TOO_LARGE;
    if (count == 1) {
        std::memcpy(output, input, r.elem_bytes);
        return RSBD8G_OK;
    }
    if (device_bytes == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            cudaGetLastError();
            return RSBD8G_ERR_CUDA;
        }
        device_bytes = fr / 10 * 9;
    }
    return chunked_sort(r, count, input, output, device_bytes, reinterpret_cast<cudaStream_t>(stream));
}

}  // extern "C"
