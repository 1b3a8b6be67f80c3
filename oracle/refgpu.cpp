// refgpu.cpp -- launch the REFERENCE's own GPU kernel (mcKernel) on this GPU.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles the reference's
// src/anneal_kernels.cu device code, unchanged, into
// oracle/_ref/anneal_kernels.cubin; this harness loads that cubin with the
// CUDA driver API, finds the requested mcKernel<SType, kPacked, kCorr>
// instantiation by enumerating the module's functions, and launches it with
// buffers laid out the way the reference's host driver prepares them
// (src/anneal_kernels.cu:612-831: per-chain slices of stride nPad = n rounded
// up to 8, winnerGroup preset to -1, AnnealState seeded with the initial cut,
// run-length beta tables, dynamic shared memory 5*maxP*8 + tpb*8 + maxP*4 +
// (2*maxP+1)*4, tpb clamped to the instantiation's limit).  Used to pin this
// project's kernel against the reference kernel bit for bit and to time the
// plain one-graph-per-launch kernel on the same GPU.  Never shipped.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct DevCsrArg {          // the reference's DevCsr (src/anneal_gpu.cuh:23-28)
    const uint32_t* offsets;
    const int32_t* edgeTo;
    const int32_t* edgeWeight;
    int64_t n;
};

struct AnnealStateArg {     // the reference's AnnealState (src/anneal_gpu.cuh:32-37)
    int64_t currentVal;
    int64_t bestVal;
    int32_t improved;
    int32_t pad;
};

struct Err {
    char* buf;
    int len;
    int set(const char* what, int code) {
        if (buf && len > 0) std::snprintf(buf, len, "%s failed (%d)", what, code);
        return code ? code : -1;
    }
};

#define DRV(call)                                         \
    do {                                                  \
        CUresult r_ = (call);                             \
        if (r_ != CUDA_SUCCESS) return e.set(#call, r_);  \
    } while (0)
#define RT(call)                                          \
    do {                                                  \
        cudaError_t r_ = (call);                          \
        if (r_ != cudaSuccess) return e.set(#call, r_);   \
    } while (0)

template <class T>
struct Buf {
    T* p = nullptr;
    ~Buf() { if (p) cudaFree(p); }
};

}  // namespace

extern "C" int refgpu_run(const char* cubin, int s64, int packed, int corrWarp, int tpb,
                          int64_t n, const uint32_t* offsets, const int32_t* col,
                          const int32_t* weight, int64_t C, const int8_t* initSpins,
                          const int64_t* initCut, int64_t nruns, const int64_t* runEnd,
                          const int32_t* runVal, const int64_t* chainOff,
                          const uint64_t* solverSeeds, int64_t nphases, const uint64_t* phases,
                          const uint64_t* iters, int8_t* endSpins, int8_t* bestSpins,
                          int64_t* curOut, int64_t* bestOut, float* ms, int* tpbUsed,
                          char* errbuf, int errlen) {
    Err e{errbuf, errlen};
    RT(cudaFree(nullptr));   // create the primary context
    CUmodule mod;
    DRV(cuModuleLoad(&mod, cubin));
    unsigned int count = 0;
    DRV(cuModuleGetFunctionCount(&count, mod));
    std::vector<CUfunction> fns(count);
    DRV(cuModuleEnumerateFunctions(fns.data(), count, mod));
    // mcKernel<SType, kPacked, kCorr>: template args mangle as
    // I{i|l}Lb{0|1}ELNS_8CorrModeE{0|1}E
    const std::string want = std::string("mcKernelI") + (s64 ? "l" : "i") + "Lb" +
                             (packed ? "1" : "0") + "ELNS_8CorrModeE" + (corrWarp ? "1" : "0") + "E";
    CUfunction f = nullptr;
    for (CUfunction c : fns) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, c) == CUDA_SUCCESS && name && std::strstr(name, want.c_str())) f = c;
    }
    if (!f) { cuModuleUnload(mod); return e.set("kernel lookup", -2); }
    DRV(cuFuncLoad(f));   // enumerated functions are not loaded under lazy loading

    const int64_t nPad = (n + 7) & ~int64_t{7};
    const int64_t m2 = offsets[n];
    int64_t maxP = 0;
    for (int64_t p = 0; p < nphases; ++p) maxP = std::max<int64_t>(maxP, static_cast<int64_t>(phases[p]));
    int maxThreads = 0;
    DRV(cuFuncGetAttribute(&maxThreads, CU_FUNC_ATTRIBUTE_MAX_THREADS_PER_BLOCK, f));
    const int t = std::min(tpb, maxThreads);
    *tpbUsed = t;
    const size_t smem = static_cast<size_t>(maxP) * 5 * 8 + static_cast<size_t>(t) * 8 +
                        static_cast<size_t>(maxP) * 4 + (2 * static_cast<size_t>(maxP) + 1) * 4;
    DRV(cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, static_cast<int>(smem)));

    const size_t sBytes = s64 ? 8 : 4;
    Buf<uint32_t> dOff;
    Buf<int32_t> dTo, dW, dWG, dRunVal;
    Buf<int8_t> dSpin, dBest;
    Buf<unsigned char> dS;
    Buf<int64_t> dRunEnd, dChainOff;
    Buf<uint64_t> dSeeds, dPhaseP, dPhaseIters;
    Buf<AnnealStateArg> dSt;
    RT(cudaMalloc(&dOff.p, (n + 1) * 4));
    RT(cudaMalloc(&dTo.p, std::max<int64_t>(m2, 1) * 4));
    RT(cudaMalloc(&dW.p, std::max<int64_t>(m2, 1) * 4));
    RT(cudaMalloc(&dSpin.p, C * nPad));
    RT(cudaMalloc(&dBest.p, C * nPad));
    RT(cudaMalloc(&dS.p, C * nPad * sBytes));
    RT(cudaMalloc(&dWG.p, C * nPad * 4));
    RT(cudaMalloc(&dSt.p, C * sizeof(AnnealStateArg)));
    RT(cudaMalloc(&dRunEnd.p, nruns * 8));
    RT(cudaMalloc(&dRunVal.p, nruns * 4));
    RT(cudaMalloc(&dChainOff.p, C * 8));
    RT(cudaMalloc(&dSeeds.p, C * 8));
    RT(cudaMalloc(&dPhaseP.p, std::max<int64_t>(nphases, 1) * 8));
    RT(cudaMalloc(&dPhaseIters.p, std::max<int64_t>(nphases, 1) * 8));
    RT(cudaMemset(dS.p, 0, C * nPad * sBytes));
    RT(cudaMemset(dWG.p, 0xFF, C * nPad * 4));
    RT(cudaMemcpy(dOff.p, offsets, (n + 1) * 4, cudaMemcpyHostToDevice));
    if (m2) {
        RT(cudaMemcpy(dTo.p, col, m2 * 4, cudaMemcpyHostToDevice));
        RT(cudaMemcpy(dW.p, weight, m2 * 4, cudaMemcpyHostToDevice));
    }
    std::vector<int8_t> hs(static_cast<size_t>(C * nPad), 0);
    for (int64_t c = 0; c < C; ++c) std::memcpy(&hs[c * nPad], initSpins + c * n, n);
    RT(cudaMemcpy(dSpin.p, hs.data(), hs.size(), cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dBest.p, hs.data(), hs.size(), cudaMemcpyHostToDevice));
    std::vector<AnnealStateArg> st(C);
    for (int64_t c = 0; c < C; ++c) st[c] = AnnealStateArg{initCut[c], initCut[c], 0, 0};
    RT(cudaMemcpy(dSt.p, st.data(), C * sizeof(AnnealStateArg), cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dRunEnd.p, runEnd, nruns * 8, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dRunVal.p, runVal, nruns * 4, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dChainOff.p, chainOff, C * 8, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(dSeeds.p, solverSeeds, C * 8, cudaMemcpyHostToDevice));
    if (nphases) {
        RT(cudaMemcpy(dPhaseP.p, phases, nphases * 8, cudaMemcpyHostToDevice));
        RT(cudaMemcpy(dPhaseIters.p, iters, nphases * 8, cudaMemcpyHostToDevice));
    }

    DevCsrArg g{dOff.p, dTo.p, dW.p, n};
    int8_t* a1 = dSpin.p;
    int8_t* a2 = dBest.p;
    void* a3 = dS.p;
    const int64_t* a4 = dRunEnd.p;
    const int32_t* a5 = dRunVal.p;
    const int64_t* a6 = dChainOff.p;
    const uint64_t* a7 = dPhaseP.p;
    const uint64_t* a8 = dPhaseIters.p;
    int64_t a9 = nphases;
    const uint64_t* a10 = dSeeds.p;
    AnnealStateArg* a11 = dSt.p;
    int64_t a12 = maxP;
    int32_t* a13 = dWG.p;
    int64_t a14 = nPad;
    void* params[] = {&g, &a1, &a2, &a3, &a4, &a5, &a6, &a7, &a8, &a9, &a10, &a11, &a12, &a13, &a14};
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    RT(cudaEventRecord(e0, 0));
    DRV(cuLaunchKernel(f, static_cast<unsigned>(C), 1, 1, t, 1, 1, static_cast<unsigned>(smem),
                       nullptr, params, nullptr));
    RT(cudaEventRecord(e1, 0));
    RT(cudaEventSynchronize(e1));
    RT(cudaGetLastError());
    RT(cudaEventElapsedTime(ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);

    std::vector<int8_t> he(hs.size()), hb(hs.size());
    RT(cudaMemcpy(he.data(), dSpin.p, he.size(), cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(hb.data(), dBest.p, hb.size(), cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(st.data(), dSt.p, C * sizeof(AnnealStateArg), cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < C; ++c) {
        std::memcpy(endSpins + c * n, &he[c * nPad], n);
        std::memcpy(bestSpins + c * n, &hb[c * nPad], n);
        curOut[c] = st[c].currentVal;
        bestOut[c] = st[c].bestVal;
    }
    cuModuleUnload(mod);
    return 0;
}
