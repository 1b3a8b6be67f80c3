// rfmf_ingest.cu -- graph ingest and output path of librfmf.so.
//
// Ingest (reference: src/read_gset.cpp:61-201 parseAndScale +
// read_instance_from_stream, src/graph.cpp addEdge, src/immutable_graph.hpp:
// 44-120 ImmutableGraph::build):
//   * rfmf_gset_header / rfmf_gset_parse: native parser of Gset/MQLib text
//     with the reference's rules (comment and blank lines skipped, header
//     "N M", M edge lines "u v w", power-of-ten scaling when a weight is
//     fractional, zero weights dropped after rounding);
//   * rfmf_graph_from_edges: the CSR built ON THE DEVICE from an edge list --
//     undirected duplicates keep their first weight, vertices are the
//     endpoints of the surviving edges renumbered densely in ascending
//     original id, every row sorted ascending -- then the compact shared-memory
//     entry formats, B and the weight sum, all without a host CSR.
//     Steps: endpoint presence marks and an exclusive scan give the dense ids;
//     a degree histogram and scan give row starts; entries scatter to their
//     rows tagged with their input index; each row is sorted by (neighbour,
//     input index) so the first occurrence of a duplicate leads its run;
//     runs collapse to their first entry and the rows compact.
// Output (reference: src/max_cut.cpp:5-15 cutValueCsr and the
// Solution-*-partition: lines of src/host_common.cpp:412-422):
//   * rfmf_batch_cuts: every chain's cut recomputed on the device from its
//     end or best spins;
//   * rfmf_batch_partitions: the '0'/'1' partition strings of every chain
//     expanded on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <utility>
#include <vector>

#include "rfmf_host.h"

using namespace rfmf;

// ======================================================================
// Gset / MQLib text parser (host)
// ======================================================================
// The text format and the weight rule this parser implements (the loader
// behaviour of src/read_gset.cpp:61-170, restated):
//   * lines end at '\n'; a line that is empty after leading spaces, tabs and
//     CRs, or whose first such character is '#', carries no data;
//   * the first data line holds N and M (integers >= 0), the next M data
//     lines one edge each: two integer ids and a real weight, any further
//     text on the line ignored;
//   * weights that are all integral (w == floor(w), |w| < 2^53) are used
//     as they are.  Otherwise every weight is multiplied by one power of
//     ten s = 10^k, k in 12..-12, the largest for which A s + D / 2 stays
//     within a budget and W s within (2^31 - 1) / 2, where W is the largest
//     |w|, and over the ids of the edge lines, A the largest sum of |w| of
//     an id's lines and D the largest number of line ends at one id.  The
//     budget is (2^31 - 1) / 4, or (2^63 - 1) / 8 when no k meets the first;
//     no k at all, or W s < 1/2 (every weight would round to zero), is an
//     error.  Scaled weights are rounded to the nearest integer, halves away
//     from zero;
//   * edges whose integer weight is 0 are dropped and counted; the others
//     are returned in file order, duplicates included.
// A forced scale s > 0 replaces the choice and its two checks.
namespace {

// Data lines of the text as [begin, end) spans, in order.
std::vector<std::pair<const char*, const char*>> data_lines(const char* text, size_t len) {
    std::vector<std::pair<const char*, const char*>> out;
    const char* const stop = text + len;
    for (const char* cur = text; cur < stop;) {
        const char* nl = static_cast<const char*>(std::memchr(cur, '\n', static_cast<size_t>(stop - cur)));
        const char* lineEnd = nl ? nl : stop;
        const char* first = cur;
        while (first < lineEnd && (*first == ' ' || *first == '\t' || *first == '\r')) ++first;
        if (first < lineEnd && *first != '#') out.emplace_back(cur, lineEnd);
        cur = nl ? nl + 1 : stop;
    }
    return out;
}

// Reads numbers off one line (a NUL-terminated copy, so the C library
// conversions stop at its end).
class LineScanner {
public:
    LineScanner(const char* b, const char* e) : text_(b, e) { text_.push_back('\0'); at_ = text_.data(); }
    bool integer(long long& x) {
        char* after = nullptr;
        x = std::strtoll(at_, &after, 10);
        return advance(after);
    }
    bool real(double& x) {
        char* after = nullptr;
        x = std::strtod(at_, &after);
        return advance(after);
    }

private:
    bool advance(char* after) {
        if (after == at_) return false;
        at_ = after;
        return true;
    }
    std::vector<char> text_;
    const char* at_;
};

struct EdgeLine {
    int64_t a, b;
    double w;
};

bool whole_number(double w) { return w == std::floor(w) && std::fabs(w) < 9007199254740992.0; }

// W, A and D of the weight rule over the edge lines.  Each line contributes
// (id, |w|) for both of its ends; a stable sort by id keeps every id's
// contributions in file order, so each per-id sum is accumulated in line
// order.
struct WeightBounds {
    double maxAbs = 0.0, maxIdSum = 0.0, maxIdEnds = 0.0;
};

WeightBounds weight_bounds(const std::vector<EdgeLine>& lines) {
    WeightBounds wb;
    std::vector<std::pair<int64_t, double>> ends;
    ends.reserve(2 * lines.size());
    for (const EdgeLine& l : lines) {
        const double mag = std::fabs(l.w);
        wb.maxAbs = std::max(wb.maxAbs, mag);
        ends.emplace_back(l.a, mag);
        ends.emplace_back(l.b, mag);
    }
    std::stable_sort(ends.begin(), ends.end(),
                     [](const std::pair<int64_t, double>& x, const std::pair<int64_t, double>& y) {
                         return x.first < y.first;
                     });
    for (size_t lo = 0; lo < ends.size();) {
        size_t hi = lo;
        double sum = 0.0;
        for (; hi < ends.size() && ends[hi].first == ends[lo].first; ++hi) sum += ends[hi].second;
        wb.maxIdSum = std::max(wb.maxIdSum, sum);
        wb.maxIdEnds = std::max(wb.maxIdEnds, static_cast<double>(hi - lo));
        lo = hi;
    }
    return wb;
}

// The power of ten of the weight rule, or 0 when none qualifies.
double power_of_ten_scale(const WeightBounds& wb) {
    static const double kPow10[25] = {1e12, 1e11, 1e10, 1e9,  1e8,   1e7,   1e6,   1e5,  1e4,
                                      1e3,  1e2,  1e1,  1e0,  1e-1,  1e-2,  1e-3,  1e-4, 1e-5,
                                      1e-6, 1e-7, 1e-8, 1e-9, 1e-10, 1e-11, 1e-12};
    const double weightCap = static_cast<double>(std::numeric_limits<int32_t>::max()) / 2;
    const double sumCaps[2] = {static_cast<double>(std::numeric_limits<int32_t>::max()) / 4,
                               static_cast<double>(std::numeric_limits<int64_t>::max()) / 8};
    for (double cap : sumCaps)
        for (double s : kPow10)
            if (wb.maxIdSum * s + wb.maxIdEnds / 2 <= cap && wb.maxAbs * s <= weightCap) return s;
    return 0.0;
}

}  // namespace

extern "C" int rfmf_gset_header(const char* text, size_t len, int64_t* n, int64_t* m) {
    if (!text || !n || !m) return fail(RFMF_ERR_INVALID, "text/n/m is NULL");
    const auto lines = data_lines(text, len);
    long long N = -1, M = -1;
    if (lines.empty()) return fail(RFMF_ERR_INVALID, "no data line: the first must hold the vertex and edge counts");
    LineScanner sc(lines[0].first, lines[0].second);
    if (!sc.integer(N) || !sc.integer(M) || N < 0 || M < 0)
        return fail(RFMF_ERR_INVALID, "the first data line must hold two counts >= 0 (vertices, edges)");
    *n = N;
    *m = M;
    return RFMF_OK;
}

static int rfmf_gset_parse_impl(const char* text, size_t len, double forced_scale, int64_t cap,
                               int64_t* u, int64_t* v, int64_t* w, int64_t* nedges,
                               double* scale_out, int64_t* zero_dropped) {
    if (!text || !u || !v || !w || !nedges) return fail(RFMF_ERR_INVALID, "NULL argument");
    host_alloc_point();
    int64_t N = 0, M = 0;
    if (int rc = rfmf_gset_header(text, len, &N, &M)) return rc;
    if (cap < M) return fail(RFMF_ERR_CAPACITY, "cap %lld < %lld edges", (long long)cap, (long long)M);
    const auto lines = data_lines(text, len);
    if (static_cast<int64_t>(lines.size()) - 1 < M)
        return fail(RFMF_ERR_INVALID, "header announces %lld edges, the text has %lld edge lines",
                    (long long)M, (long long)(lines.size() - 1));
    std::vector<EdgeLine> edges(static_cast<size_t>(M));
    bool allWhole = true;
    for (int64_t i = 0; i < M; ++i) {
        LineScanner sc(lines[i + 1].first, lines[i + 1].second);
        long long a = 0, b = 0;
        double x = 0.0;
        if (!sc.integer(a) || !sc.integer(b) || !sc.real(x))
            return fail(RFMF_ERR_INVALID, "edge line %lld: expected two ids and a weight", (long long)i);
        edges[i] = EdgeLine{a, b, x};
        allWhole = allWhole && whole_number(x);
    }
    double s = 1.0;
    if (forced_scale > 0.0) {
        s = forced_scale;
    } else if (!allWhole) {
        const WeightBounds wb = weight_bounds(edges);
        s = power_of_ten_scale(wb);
        if (s == 0.0)
            return fail(RFMF_ERR_INVALID, "weights too large for any power-of-ten scale (max |w| %g, max id |w| sum %g)",
                        wb.maxAbs, wb.maxIdSum);
        if (wb.maxAbs * s < 0.5)
            return fail(RFMF_ERR_INVALID, "at scale %g every weight rounds to zero (max |w| %g)", s, wb.maxAbs);
    }
    int64_t kept = 0, zeros = 0;
    for (const EdgeLine& l : edges) {
        const int64_t iw = (s == 1.0 && whole_number(l.w)) ? static_cast<int64_t>(l.w) : std::llround(l.w * s);
        if (iw == 0) {
            ++zeros;
            continue;
        }
        u[kept] = l.a;
        v[kept] = l.b;
        w[kept] = iw;
        ++kept;
    }
    *nedges = kept;
    if (scale_out) *scale_out = s;
    if (zero_dropped) *zero_dropped = zeros;
    return RFMF_OK;
}

// ======================================================================
// CSR build on the device
// ======================================================================
namespace {

constexpr int kScanBlock = 1024;     // threads per scan block
constexpr int kScanItems = 4;        // items per thread
constexpr int kScanTile = kScanBlock * kScanItems;

// Exclusive scan of one tile per block; the block total goes to sums[block].
template <class T>
__global__ void scan_tiles(const T* in, T* out, T* sums, int64_t n) {
    __shared__ T warpTot[kScanBlock / 32];
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
    T v[kScanItems];
    T run = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : T(0);
        const T x = v[k];
        v[k] = run;
        run += x;
    }
    // inclusive warp scan of the thread totals
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const T o = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= d) incl += o;
    }
    if (lane == 31) warpTot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        T t = (lane < kScanBlock / 32) ? warpTot[lane] : T(0);
        T ti = t;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const T o = __shfl_up_sync(0xFFFFFFFFu, ti, d);
            if (lane >= d) ti += o;
        }
        if (lane < kScanBlock / 32) warpTot[lane] = ti - t;   // exclusive
        if (lane == kScanBlock / 32 - 1 && sums) sums[blockIdx.x] = ti;
    }
    __syncthreads();
    const T off = warpTot[wid] + (incl - run);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) out[base + k] = v[k] + off;
}

template <class T>
__global__ void add_tile_offsets(T* out, const T* offs, int64_t n) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * kScanTile + threadIdx.x;
    const T o = offs[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t j = i + static_cast<int64_t>(k) * kScanBlock;
        if (j < n) out[j] += o;
    }
}

// Exclusive scan of n values (out may equal in), recursive over tiles.
template <class T>
int exclusive_scan(const T* in, T* out, int64_t n, cudaStream_t st) {
    if (n <= 0) return RFMF_OK;
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    DevBuf sums;
    if (int rc = sums.alloc(static_cast<size_t>(tiles + 1) * sizeof(T))) return rc;
    scan_tiles<T><<<static_cast<unsigned>(tiles), kScanBlock, 0, st>>>(in, out, sums.as<T>(), n);
    CU(cudaGetLastError());
    if (tiles > 1) {
        if (int rc = exclusive_scan<T>(sums.as<T>(), sums.as<T>(), tiles, st)) return rc;
        add_tile_offsets<T><<<static_cast<unsigned>(tiles), kScanBlock, 0, st>>>(out, sums.as<T>(), n);
        CU(cudaGetLastError());
    }
    CU(cudaStreamSynchronize(st));
    return RFMF_OK;
}

struct BuildFlags {
    int selfLoop;
    int badId;
    int notUnit;
    int notSmall;
    unsigned long long B;
    long long wsum2;
};

__global__ void mark_endpoints(const int64_t* u, const int64_t* v, int64_t E, int64_t maxId,
                               int32_t* present, BuildFlags* f) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < E;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t a = u[i], b = v[i];
        if (a < 0 || b < 0 || a > maxId || b > maxId) { atomicOr(&f->badId, 1); continue; }
        if (a == b) { atomicOr(&f->selfLoop, 1); continue; }
        present[a] = 1;
        present[b] = 1;
    }
}

__global__ void count_degrees(const int64_t* u, const int64_t* v, int64_t E, const int32_t* dense,
                              int32_t* deg) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < E;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        atomicAdd(&deg[dense[u[i]]], 1);
        atomicAdd(&deg[dense[v[i]]], 1);
    }
}

// Raw directed entry: neighbour, weight, input edge index.
struct RawEntry {
    int32_t col;
    int32_t w;
    int64_t idx;
};

__global__ void scatter_entries(const int64_t* u, const int64_t* v, const int64_t* w, int64_t E,
                                const int32_t* dense, const int32_t* rowStart, int32_t* fill,
                                RawEntry* ent) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < E;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t a = dense[u[i]], b = dense[v[i]];
        const int32_t wi = static_cast<int32_t>(w[i]);
        const int32_t pa = rowStart[a] + atomicAdd(&fill[a], 1);
        const int32_t pb = rowStart[b] + atomicAdd(&fill[b], 1);
        ent[pa] = RawEntry{b, wi, i};
        ent[pb] = RawEntry{a, wi, i};
    }
}

// One thread per row: insertion sort by (col, idx); then the first entry of
// each col run survives.  Writes the surviving count of the row.
__global__ void sort_rows(RawEntry* ent, const int32_t* rowStart, int32_t n, int32_t* keep) {
    for (int32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int32_t lo = rowStart[r], hi = rowStart[r + 1];
        for (int32_t i = lo + 1; i < hi; ++i) {
            const RawEntry x = ent[i];
            int32_t j = i - 1;
            while (j >= lo && (ent[j].col > x.col || (ent[j].col == x.col && ent[j].idx > x.idx))) {
                ent[j + 1] = ent[j];
                --j;
            }
            ent[j + 1] = x;
        }
        int32_t k = 0;
        for (int32_t i = lo; i < hi; ++i)
            if (i == lo || ent[i].col != ent[i - 1].col) ++k;
        keep[r] = k;
    }
}

__global__ void compact_rows(const RawEntry* ent, const int32_t* rowStart, const int32_t* outStart,
                             int32_t n, uint32_t* offsets, Edge* edges, BuildFlags* f) {
    for (int32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int32_t lo = rowStart[r], hi = rowStart[r + 1];
        int32_t o = outStart[r];
        offsets[r] = static_cast<uint32_t>(o);
        long long b = 0, s = 0;
        bool unit = true, small = true;
        for (int32_t i = lo; i < hi; ++i) {
            if (i != lo && ent[i].col == ent[i - 1].col) continue;
            const int32_t wi = ent[i].w;
            edges[o++] = Edge{ent[i].col, wi};
            b += (wi < 0) ? -static_cast<long long>(wi) : wi;
            s += wi;
            unit = unit && (wi == 1 || wi == -1);
            small = small && (wi >= -32767 && wi <= 32767);
        }
        atomicMax(&f->B, static_cast<unsigned long long>(b));
        atomicAdd(reinterpret_cast<unsigned long long*>(&f->wsum2), static_cast<unsigned long long>(s));
        if (!unit) atomicOr(&f->notUnit, 1);
        if (!small) atomicOr(&f->notSmall, 1);
    }
}

__global__ void orig_ids(const int32_t* present, const int32_t* dense, int64_t maxId, int64_t* out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i <= maxId;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        if (present[i]) out[dense[i]] = i;
}

__global__ void make_compact(const Edge* edges, int64_t m2, int fmt, void* out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < m2;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const Edge e = edges[i];
        if (fmt == kCsrUnit16)
            static_cast<uint16_t*>(out)[i] =
                static_cast<uint16_t>((static_cast<uint32_t>(e.col) << 1) | (e.w < 0 ? 1u : 0u));
        else
            static_cast<uint32_t*>(out)[i] = (static_cast<uint32_t>(e.w) << 16) | static_cast<uint32_t>(e.col);
    }
}

__global__ void fill_tail_u32(uint32_t* p, int64_t from, int64_t to, uint32_t val) {
    for (int64_t i = from + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < to;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        p[i] = val;
}

unsigned grid_for(int64_t n) {
    return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4096)));
}

}  // namespace

static int rfmf_graph_from_edges_impl(rfmf_context* ctx, int64_t nedges, const int64_t* u,
                                     const int64_t* v, const int64_t* w, rfmf_graph** out,
                                     int64_t* n_out) {
    if (!ctx || !out || nedges < 0 || (nedges > 0 && (!u || !v || !w)))
        return fail(RFMF_ERR_INVALID, "bad arguments");
    *out = nullptr;
    // Zero weights drop (the parser's rule); ids and weights checked.
    std::vector<int64_t> hu, hv, hw;
    hu.reserve(static_cast<size_t>(nedges));
    hv.reserve(static_cast<size_t>(nedges));
    hw.reserve(static_cast<size_t>(nedges));
    int64_t maxId = 0;
    for (int64_t i = 0; i < nedges; ++i) {
        if (u[i] < 0 || v[i] < 0) return fail(RFMF_ERR_INVALID, "negative vertex id at edge %lld", (long long)i);
        if (w[i] == 0) continue;
        if (w[i] > std::numeric_limits<int32_t>::max() || w[i] < -std::numeric_limits<int32_t>::max())
            return fail(RFMF_ERR_CAPACITY, "weight at edge %lld does not fit int32", (long long)i);
        maxId = std::max(maxId, std::max(u[i], v[i]));
        hu.push_back(u[i]);
        hv.push_back(v[i]);
        hw.push_back(w[i]);
    }
    const int64_t E = static_cast<int64_t>(hu.size());
    if (maxId >= (int64_t(1) << 28))
        return fail(RFMF_ERR_CAPACITY, "vertex ids up to %lld: the device build takes ids below 2^28",
                    (long long)maxId);
    if (2 * E >= (int64_t(1) << 31)) return fail(RFMF_ERR_CAPACITY, "too many edges");
    CU(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t ids = maxId + 1;
    DevBuf dU, dV, dW, dPresent, dDense, dFlags;
    int rc;
    if ((rc = dU.alloc(E * 8)) || (rc = dV.alloc(E * 8)) || (rc = dW.alloc(E * 8)) ||
        (rc = dPresent.alloc((ids + 1) * 4)) || (rc = dDense.alloc((ids + 1) * 4)) ||
        (rc = dFlags.alloc(sizeof(BuildFlags))))
        return rc;
    if (E) {
        CU(cudaMemcpyAsync(dU.p, hu.data(), E * 8, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(dV.p, hv.data(), E * 8, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(dW.p, hw.data(), E * 8, cudaMemcpyHostToDevice, st));
    }
    CU(cudaMemsetAsync(dPresent.p, 0, (ids + 1) * 4, st));
    CU(cudaMemsetAsync(dFlags.p, 0, sizeof(BuildFlags), st));
    if (E) mark_endpoints<<<grid_for(E), 256, 0, st>>>(dU.as<int64_t>(), dV.as<int64_t>(), E, maxId,
                                                       dPresent.as<int32_t>(), dFlags.as<BuildFlags>());
    CU(cudaGetLastError());
    // dense ids: exclusive scan of presence over ids + 1 slots; n = last value
    if ((rc = exclusive_scan<int32_t>(dPresent.as<int32_t>(), dDense.as<int32_t>(), ids + 1, st)))
        return rc;
    BuildFlags hf{};
    int32_t n32 = 0;
    CU(cudaMemcpyAsync(&hf, dFlags.p, sizeof hf, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&n32, dDense.as<int32_t>() + ids, 4, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (hf.selfLoop) return fail(RFMF_ERR_INVALID, "self loop in the edge list");
    const int32_t n = n32;
    // degrees and row starts (n + 1 slots; slot n becomes 2E)
    DevBuf dDeg, dRow, dFill, dEnt, dKeep, dOut;
    if ((rc = dDeg.alloc((static_cast<int64_t>(n) + 1) * 4)) || (rc = dRow.alloc((static_cast<int64_t>(n) + 1) * 4)) ||
        (rc = dFill.alloc((static_cast<int64_t>(n) + 1) * 4)) || (rc = dEnt.alloc(std::max<int64_t>(2 * E, 1) * sizeof(RawEntry))) ||
        (rc = dKeep.alloc((static_cast<int64_t>(n) + 1) * 4)) || (rc = dOut.alloc((static_cast<int64_t>(n) + 1) * 4)))
        return rc;
    CU(cudaMemsetAsync(dDeg.p, 0, (static_cast<int64_t>(n) + 1) * 4, st));
    CU(cudaMemsetAsync(dFill.p, 0, (static_cast<int64_t>(n) + 1) * 4, st));
    CU(cudaMemsetAsync(dKeep.p, 0, (static_cast<int64_t>(n) + 1) * 4, st));
    if (E) count_degrees<<<grid_for(E), 256, 0, st>>>(dU.as<int64_t>(), dV.as<int64_t>(), E,
                                                      dDense.as<int32_t>(), dDeg.as<int32_t>());
    CU(cudaGetLastError());
    if ((rc = exclusive_scan<int32_t>(dDeg.as<int32_t>(), dRow.as<int32_t>(), static_cast<int64_t>(n) + 1, st)))
        return rc;
    if (E) scatter_entries<<<grid_for(E), 256, 0, st>>>(dU.as<int64_t>(), dV.as<int64_t>(), dW.as<int64_t>(), E,
                                                        dDense.as<int32_t>(), dRow.as<int32_t>(),
                                                        dFill.as<int32_t>(), dEnt.as<RawEntry>());
    CU(cudaGetLastError());
    if (n) sort_rows<<<grid_for(n), 256, 0, st>>>(dEnt.as<RawEntry>(), dRow.as<int32_t>(), n, dKeep.as<int32_t>());
    CU(cudaGetLastError());
    if ((rc = exclusive_scan<int32_t>(dKeep.as<int32_t>(), dOut.as<int32_t>(), static_cast<int64_t>(n) + 1, st)))
        return rc;
    int32_t m2 = 0;
    CU(cudaMemcpyAsync(&m2, dOut.as<int32_t>() + n, 4, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));

    auto g = std::unique_ptr<rfmf_graph>(new (std::nothrow) rfmf_graph());
    if (!g) return fail(RFMF_ERR_NOMEM, "host allocation failed");
    g->ctxHold.set(ctx);
    g->ctx = ctx;
    g->n = n;
    g->m = m2 / 2;
    const uint64_t ob = (static_cast<uint64_t>(n + 1) * 4u + 15u) & ~uint64_t(15);
    g->offBytes = static_cast<uint32_t>(ob);
    if ((rc = g->offsets.alloc(ob)) || (rc = g->edges.alloc(std::max<int64_t>(m2, 1) * sizeof(Edge)))) return rc;
    if (n) compact_rows<<<grid_for(n), 256, 0, st>>>(dEnt.as<RawEntry>(), dRow.as<int32_t>(), dOut.as<int32_t>(), n,
                                                     g->offsets.as<uint32_t>(), g->edges.as<Edge>(),
                                                     dFlags.as<BuildFlags>());
    CU(cudaGetLastError());
    // offsets[n .. padded end] = m2
    fill_tail_u32<<<1, 256, 0, st>>>(g->offsets.as<uint32_t>(), n, static_cast<int64_t>(ob / 4), static_cast<uint32_t>(m2));
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(&hf, dFlags.p, sizeof hf, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    g->B = static_cast<int64_t>(hf.B);
    g->wsum2 = hf.wsum2;
    if (g->B > std::numeric_limits<int32_t>::max())
        return fail(RFMF_ERR_CAPACITY, "max weighted degree %lld exceeds int32", (long long)g->B);
    g->unit16 = !hf.notUnit && n <= 32768;
    g->packed32 = !hf.notSmall && n <= 65536 && m2 < (1 << 30);
    if (g->unit16) {
        g->u16Bytes = align16(static_cast<uint32_t>(m2) * 2u);
        if ((rc = g->u16.alloc(g->u16Bytes))) return rc;
        CU(cudaMemsetAsync(g->u16.p, 0, g->u16Bytes, st));
        if (m2) make_compact<<<grid_for(m2), 256, 0, st>>>(g->edges.as<Edge>(), m2, kCsrUnit16, g->u16.p);
    }
    if (g->packed32) {
        g->p32Bytes = align16(static_cast<uint32_t>(m2) * 4u);
        if ((rc = g->p32.alloc(g->p32Bytes))) return rc;
        CU(cudaMemsetAsync(g->p32.p, 0, g->p32Bytes, st));
        if (m2) make_compact<<<grid_for(m2), 256, 0, st>>>(g->edges.as<Edge>(), m2, kCsrPacked32, g->p32.p);
    }
    CU(cudaGetLastError());
    // dense id -> original id, kept on the host with the graph
    {
        DevBuf dIds;
        if ((rc = dIds.alloc(std::max<int64_t>(n, 1) * 8))) return rc;
        if (n) orig_ids<<<grid_for(ids), 256, 0, st>>>(dPresent.as<int32_t>(), dDense.as<int32_t>(), maxId,
                                                       dIds.as<int64_t>());
        CU(cudaGetLastError());
        g->origIds.resize(static_cast<size_t>(n));
        if (n) CU(cudaMemcpyAsync(g->origIds.data(), dIds.p, n * 8, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
    }
    if (n_out) *n_out = n;
    *out = g.release();
    return RFMF_OK;
}

static int rfmf_graph_orig_ids_impl(const rfmf_graph* g, int64_t* out) {
    if (!g || !out) return fail(RFMF_ERR_INVALID, "graph/out is NULL");
    if (static_cast<int64_t>(g->origIds.size()) != g->n)
        return fail(RFMF_ERR_INVALID, "graph was not built from an edge list");
    std::copy(g->origIds.begin(), g->origIds.end(), out);
    return RFMF_OK;
}

static int rfmf_graph_csr_impl(const rfmf_graph* g, uint32_t* offsets, int32_t* col, int32_t* weight) {
    if (!g) return fail(RFMF_ERR_INVALID, "graph is NULL");
    CU(cudaSetDevice(g->ctx->device));
    const int64_t m2 = 2 * g->m;
    if (offsets) CU(cudaMemcpy(offsets, g->offsets.p, (g->n + 1) * 4, cudaMemcpyDeviceToHost));
    if ((col || weight) && m2) {
        std::vector<Edge> e(static_cast<size_t>(m2));
        CU(cudaMemcpy(e.data(), g->edges.p, m2 * sizeof(Edge), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < m2; ++i) {
            if (col) col[i] = e[i].col;
            if (weight) weight[i] = e[i].w;
        }
    }
    return RFMF_OK;
}

// ======================================================================
// Output path (device)
// ======================================================================
namespace {

__device__ __forceinline__ int bit_of(const uint32_t* bits, int v) {
    return (bits[v >> 5] >> (v & 31)) & 1;
}

// One CTA per chain: cutValueCsr of its end (which 0) or best (which 1)
// spins -- every directed entry (v, u) with u > v across the cut adds w.
__global__ void chain_cuts_kernel(const DevChain* chains, const DevGraph* graphs, int C, int which,
                                  int64_t* out) {
    __shared__ long long part[32];
    const int c = blockIdx.x;
    if (c >= C) return;
    const DevChain& ch = chains[c];
    const DevGraph& g = graphs[ch.graph];
    const uint32_t* bits = which ? ch.bestBits : ch.spinBits;
    long long acc = 0;
    for (int v = threadIdx.x; v < g.n; v += blockDim.x) {
        const int sv = bit_of(bits, v);
        for (uint32_t i = g.offsets[v]; i < g.offsets[v + 1]; ++i) {
            const Edge e = g.edges[i];
            if (e.col > v && bit_of(bits, e.col) != sv) acc += e.w;
        }
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, m);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += part[w];
        out[c] = t;
    }
}

// '0'/'1' per vertex of chains [c0, c0 + gridDim.y) into out (row stride).
__global__ void chain_partitions_kernel(const DevChain* chains, const DevGraph* graphs, int c0,
                                        int which, char* out, int64_t stride) {
    const int c = c0 + blockIdx.y;
    const DevChain& ch = chains[c];
    const int n = graphs[ch.graph].n;
    const uint32_t* bits = which ? ch.bestBits : ch.spinBits;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        out[static_cast<int64_t>(blockIdx.y) * stride + v] = bit_of(bits, v) ? '1' : '0';
}

}  // namespace

namespace rfmf {

cudaError_t launch_chain_cuts(const DevChain* chains, const DevGraph* graphs, int C, int which,
                              int64_t* out, cudaStream_t st) {
    if (C <= 0) return cudaSuccess;
    chain_cuts_kernel<<<C, 256, 0, st>>>(chains, graphs, C, which, out);
    return cudaGetLastError();
}

cudaError_t launch_chain_partitions(const DevChain* chains, const DevGraph* graphs, int c0, int count,
                                    int maxN, int which, char* out, int64_t stride, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const dim3 grid(static_cast<unsigned>(std::min(64, (maxN + 255) / 256)), static_cast<unsigned>(count));
    chain_partitions_kernel<<<grid, 256, 0, st>>>(chains, graphs, c0, which, out, stride);
    return cudaGetLastError();
}

}  // namespace rfmf

// C ABI entry points: no C++ exception crosses the boundary.
extern "C" int rfmf_gset_parse(const char* text, size_t len, double forced_scale, int64_t cap,
                               int64_t* u, int64_t* v, int64_t* w, int64_t* nedges,
                               double* scale_out, int64_t* zero_dropped) {
    try {
        return rfmf_gset_parse_impl(text, len, forced_scale, cap, u, v, w, nedges, scale_out, zero_dropped);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_gset_parse");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_gset_parse");
    }
}

extern "C" int rfmf_graph_from_edges(rfmf_context* ctx, int64_t nedges, const int64_t* u,
                                     const int64_t* v, const int64_t* w, rfmf_graph** out,
                                     int64_t* n_out) {
    try {
        return rfmf_graph_from_edges_impl(ctx, nedges, u, v, w, out, n_out);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_graph_from_edges");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_graph_from_edges");
    }
}

extern "C" int rfmf_graph_csr(const rfmf_graph* g, uint32_t* offsets, int32_t* col, int32_t* weight) {
    try {
        return rfmf_graph_csr_impl(g, offsets, col, weight);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_graph_csr");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_graph_csr");
    }
}

extern "C" int rfmf_graph_orig_ids(const rfmf_graph* g, int64_t* out) {
    try {
        return rfmf_graph_orig_ids_impl(g, out);
    } catch (const std::bad_alloc&) {
        return rfmf::fail(RFMF_ERR_NOMEM, "host allocation failed in rfmf_graph_orig_ids");
    } catch (...) {
        return rfmf::fail(RFMF_ERR_INVALID, "unexpected host exception in rfmf_graph_orig_ids");
    }
}
