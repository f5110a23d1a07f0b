// The fused batch of joins: host launch of batch_fused_kernel (vj_join_kernels.cuh), one
// cooperative launch per vj_join_batch call. Its own translation unit, compiled beside
// vj_join.cu, for the layouts vj_join_batch accepts.

#include "vj_join_kernels.cuh"

#include <map>
#include <mutex>
#include <tuple>

namespace vj {

namespace {

// Per (kernel, device): the dynamic shared memory already allowed (driver calls are made
// once, outside any stream capture that replays the launch later).
std::mutex g_fused_mutex;
std::map<std::tuple<const void *, int>, size_t> g_fused_smem;

int allow_smem(const void *kern, size_t smem) {
    int dev = 0;
    VJ_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_fused_mutex);
    size_t &allowed = g_fused_smem[std::make_tuple(kern, dev)];
    if (allowed >= smem) return VJ_OK;
    VJ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    VJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PROBE_THREADS, smem));
    VJ_CHECK(per_sm >= 1, VJ_ERR_UNSUPPORTED, "vj_join_batch: the fused launch does not fit an SM");
    allowed = smem;
    return VJ_OK;
}

}  // namespace

template <int KW, int PB, int HS>
int batch_fused_launch(const BatchFusedParams &F, int grid, size_t smem, cudaStream_t stream) {
    void (*kern)(BatchFusedParams) = F.passes ? batch_fused_kernel<KW, PB, HS, true> : batch_fused_kernel<KW, PB, HS, false>;
    VJ_CHECK(smem <= FUSED_SMEM, VJ_ERR_UNSUPPORTED, "vj_join_batch: %zu bytes of shared memory for the fused launch (at most %zu)", smem, FUSED_SMEM);
    VJ_TRY(allow_smem((const void *)kern, smem));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(PROBE_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    // cooperative: the launch fails rather than start with blocks that cannot be resident
    // together (the grid barriers need every block running)
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    VJ_CUDA(cudaLaunchKernelEx(&cfg, kern, F));
    return VJ_OK;
}

#define VJ_I(K, B) template int batch_fused_launch<K, B, 0>(const BatchFusedParams &, int, size_t, cudaStream_t);
VJ_I(1, 4)
VJ_I(1, 8)
VJ_I(2, 4)
VJ_I(2, 8)
VJ_I(4, 4)
VJ_I(4, 8)
VJ_I(6, 4)
VJ_I(6, 8)
VJ_I(8, 4)
VJ_I(8, 8)
#undef VJ_I

}  // namespace vj
