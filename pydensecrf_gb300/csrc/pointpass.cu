// pointpass.cu -- launchers of the mean-field point pass (pointpass.cuh):
// one instance per padded label count and thread shape, plus compile-time
// instances of the iteration's two passes and of the adjoint's splat pass.  Kept apart from meanfield.cu so
// that the instances compile in parallel with the other kernels.
#include <algorithm>

#include "pointpass.cuh"

namespace dcrf {

template <int MP, int S>
static cudaError_t pp_launch_s(const PPArgs &a, cudaStream_t s) {
    const dim3 g(a.ntiles), b(PPT<MP, S>::NT);
    if constexpr (MP >= 4) {  // the mean-field iteration passes, specialised
        if (a.mode == PP_HOT_STEP) return launch_pdl(pointpass_kernel<MP, S, PP_HOT_STEP>, g, b, a.smem_bytes, s, a);
        if (a.mode == PP_HOT_LAST) return launch_pdl(pointpass_kernel<MP, S, PP_HOT_LAST>, g, b, a.smem_bytes, s, a);
        if (a.mode == PP_HOT_SPLAT) return launch_pdl(pointpass_kernel<MP, S, PP_HOT_SPLAT>, g, b, a.smem_bytes, s, a);
    }
    return launch_pdl(pointpass_kernel<MP, S>, g, b, a.smem_bytes, s, a);
}

template <int MP>
static cudaError_t pp_launch(const PPArgs &a, cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (a.mode & (PP_NORM | PP_FILTER)) return launch_slice(a, MP, s);
    if constexpr (MP % 8 == 0) {
        if (a.split == 2) return pp_launch_s<MP, 2>(a, s);
    }
    return pp_launch_s<MP, 1>(a, s);
}

// Opts a point-pass instance into the largest dynamic shared memory a CTA can
// have next to its static shared memory; each launch asks for what its plan needs.
template <typename K>
static void pp_optin(K kernel) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess || optin <= 0) {
        cudaGetLastError();
        return;
    }
    const int dyn = std::min<int>(POINTPASS_SMEM_MAX, optin - (int)fa.sharedSizeBytes);
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess)
        cudaGetLastError();
}

template <int MP, int S>
static void pp_prepare_s() {
    pp_optin(pointpass_kernel<MP, S>);
    if constexpr (MP >= 4) {
        pp_optin(pointpass_kernel<MP, S, PP_HOT_STEP>);
        pp_optin(pointpass_kernel<MP, S, PP_HOT_LAST>);
        pp_optin(pointpass_kernel<MP, S, PP_HOT_SPLAT>);
    }
}

template <int MP>
static void pp_prepare() {
    pp_prepare_s<MP, 1>();
    if constexpr (MP % 8 == 0) pp_prepare_s<MP, 2>();
}

void prepare_pointpass_kernels() {
    pp_prepare<1>();
    pp_prepare<2>();
    pp_prepare<4>();
    pp_prepare<8>();
    pp_prepare<12>();
    pp_prepare<16>();
    pp_prepare<20>();
    pp_prepare<24>();
    pp_prepare<28>();
    pp_prepare<32>();
}

cudaError_t launch_pointpass(const PPArgs &a, int MP, cudaStream_t s) {
    switch (MP) {
        case 1: return pp_launch<1>(a, s);
        case 2: return pp_launch<2>(a, s);
        case 4: return pp_launch<4>(a, s);
        case 8: return pp_launch<8>(a, s);
        case 12: return pp_launch<12>(a, s);
        case 16: return pp_launch<16>(a, s);
        case 20: return pp_launch<20>(a, s);
        case 24: return pp_launch<24>(a, s);
        case 28: return pp_launch<28>(a, s);
        case 32: return pp_launch<32>(a, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace dcrf
