// A C++ caller of gpu3::annealGpu written against the reference's interface
// types, for the drop-in header's device test.  The reference declares
// anneallib::AnnealCsr (src/immutable_graph.hpp:23-160: numVertices(),
// numEdges(), neighbors(v) -> {to, weight, n}) and gpu3::LaunchConfig /
// CorrMode (src/anneal_gpu.cuh:42-58) and annealGpu's signature
// (src/anneal_gpu.cuh:76-88); this file restates just those declarations so
// that include/rfmf_annealgpu.hpp compiles and runs where the reference's
// headers are not present.  main.cu's own call (main.cu:83-85) passes the same
// arguments.
//
// Input file (little-endian): int64 n, nnz, C, nphases, B; uint32 off[n+1];
// int32 col[nnz], weight[nnz]; int8 init[C*n]; double t0s[C]; uint64
// seeds[C]; uint64 phases[nphases], iters[nphases].
// Output file: int8 end[C*n], best[C*n]; int64 bestVals[C], finalVals[C];
// float kernelMs.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace anneallib {
struct AnnealCsr {
    std::vector<uint32_t> off;
    std::vector<int32_t> to, w;
    struct NeighborSpan {
        const int32_t* to;
        const int32_t* weight;
        uint32_t n;
        uint32_t size() const { return n; }
    };
    uint64_t numVertices() const { return off.size() - 1; }
    uint64_t numEdges() const { return to.size() / 2; }
    NeighborSpan neighbors(int64_t v) const {
        return NeighborSpan{to.data() + off[v], w.data() + off[v], off[v + 1] - off[v]};
    }
};
}  // namespace anneallib

namespace gpu3 {
enum class CorrMode { Walk, Warpwalk };
struct LaunchConfig {
    CorrMode corr = CorrMode::Walk;
    int device = 0;
    int sWidth = 32;
};
void annealGpu(const anneallib::AnnealCsr& ig, int64_t maxWeightedDeg,
               const std::vector<std::vector<int8_t>>& initialSpins,
               const std::vector<double>& t0s, const std::vector<size_t>& phases,
               const std::vector<uint64_t>& iters, const std::vector<uint64_t>& solverSeeds,
               const LaunchConfig& cfg, std::vector<std::vector<int8_t>>& endSpins,
               std::vector<std::vector<int8_t>>& bestSpins, float* kernelMs,
               std::vector<int64_t>* kernelBestVals, std::vector<int64_t>* kernelFinalVals);
}  // namespace gpu3

#include "rfmf_annealgpu.hpp"

template <class T>
static void get(FILE* f, T* p, size_t count) {
    if (count && std::fread(p, sizeof(T), count, f) != count) {
        std::fprintf(stderr, "short input\n");
        std::exit(2);
    }
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s input output [drop-one-seed]\n", argv[0]);
        return 2;
    }
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int64_t hdr[5];
    get(in, hdr, 5);
    const int64_t n = hdr[0], nnz = hdr[1], C = hdr[2], np = hdr[3], B = hdr[4];
    anneallib::AnnealCsr g;
    g.off.resize(n + 1);
    g.to.resize(nnz);
    g.w.resize(nnz);
    get(in, g.off.data(), g.off.size());
    get(in, g.to.data(), g.to.size());
    get(in, g.w.data(), g.w.size());
    std::vector<std::vector<int8_t>> init(C, std::vector<int8_t>(n));
    for (auto& row : init) get(in, row.data(), row.size());
    std::vector<double> t0s(C);
    std::vector<uint64_t> seeds(C), ph64(np), iters(np);
    get(in, t0s.data(), t0s.size());
    get(in, seeds.data(), seeds.size());
    get(in, ph64.data(), ph64.size());
    get(in, iters.data(), iters.size());
    std::fclose(in);
    if (argc > 3) seeds.pop_back();   // the argument check's exit path
    std::vector<size_t> phases(ph64.begin(), ph64.end());

    gpu3::LaunchConfig cfg;
    std::vector<std::vector<int8_t>> endSpins, bestSpins;
    std::vector<int64_t> bestVals, finalVals;
    float ms = -1.0f;
    gpu3::annealGpu(g, B, init, t0s, phases, iters, seeds, cfg, endSpins, bestSpins, &ms,
                    &bestVals, &finalVals);

    FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    for (auto& row : endSpins) std::fwrite(row.data(), 1, row.size(), out);
    for (auto& row : bestSpins) std::fwrite(row.data(), 1, row.size(), out);
    std::fwrite(bestVals.data(), sizeof(int64_t), bestVals.size(), out);
    std::fwrite(finalVals.data(), sizeof(int64_t), finalVals.size(), out);
    std::fwrite(&ms, sizeof(float), 1, out);
    std::fclose(out);
    std::printf("chains %lld kernel_ms %.3f\n", static_cast<long long>(C), ms);
    return 0;
}
