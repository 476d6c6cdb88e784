// Host side of the tensor-map (TMA) loads: encoding of the row maps that the
// FFT passes load their tiles through (see tma.cuh).  The encoder is the
// driver's cuTensorMapEncodeTiled, reached through the runtime's driver
// entry-point query so that the library links against the runtime only.
#include <cudaTypedefs.h>

#include <mutex>

#include "pm_common.cuh"
#include "pm_internal.h"

namespace cpm {

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
    });
    return fn;
}

}  // namespace

cudaError_t make_row_map(CUtensorMap* map, const void* base, int rowlen, int rows, int batch, int box_rows) {
    const auto fn = encode_fn();
    if (!fn) return cudaErrorNotSupported;
    if (rowlen < 4 || (rowlen & (rowlen - 1)) != 0 || rows < box_rows || box_rows < 1 || box_rows > 256 || batch < 1)
        return cudaErrorInvalidValue;
    const uint64_t inner = rowlen < 256 ? uint64_t(rowlen) : 256u;
    const cuuint64_t dims[4] = {inner, uint64_t(rowlen) / inner, uint64_t(rows), uint64_t(batch)};
    const cuuint64_t strides[3] = {inner * 4u, uint64_t(rowlen) * 4u, uint64_t(rows) * uint64_t(rowlen) * 4u};
    const cuuint32_t box[4] = {cuuint32_t(inner), cuuint32_t(uint64_t(rowlen) / inner), cuuint32_t(box_rows), 1u};
    const cuuint32_t estr[4] = {1u, 1u, 1u, 1u};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace cpm
