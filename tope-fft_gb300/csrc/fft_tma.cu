/*
 * Tensor maps for the TMA-staged tiles of strided passes (fft_pass.cuh
 * tma_load_tile): encoded on the host with the driver's
 * cuTensorMapEncodeTiled (reached through the runtime's entry-point query,
 * so the library does not link the driver library) and copied into device
 * memory the plan owns.  A map describes the pass's array in 8-byte units:
 * dimension 0 the adjacent lines (contiguous), then the line's elements and
 * the other line dimensions ordered by stride; the box is the tile's lines
 * by up to 256 elements of the line.  No swizzle, no interleave, no L2
 * promotion; out-of-range boxes are never requested (full tiles only).
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include "tfft_abi.h"

/* the driver's encoder, looked up once (a function-local static: its
 * initialisation is thread-safe when plans are made from several threads) */
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn(void)
{
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        return nullptr;
    }();
    return fn;
}

extern "C" int tfft_tensor_map(void *dev_map, const void *base, int rank, const int64_t *dims,
                               const int64_t *strides, const int *box)
{
    if (rank < 2 || rank > 5 || ((uintptr_t)base & 15)) return (int)cudaErrorInvalidValue;
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) return (int)cudaErrorNotSupported;
    cuuint64_t gdim[5], gstride[4];
    cuuint32_t bdim[5], estride[5];
    for (int d = 0; d < rank; d++) {
        if (dims[d] < 1 || dims[d] >= ((int64_t)1 << 31) || box[d] < 1 || box[d] > 256) /* int coordinates */
            return (int)cudaErrorInvalidValue;
        gdim[d] = (cuuint64_t)dims[d];
        bdim[d] = (cuuint32_t)box[d];
        estride[d] = 1;
        if (d > 0) {
            if (strides[d - 1] % 16 || strides[d - 1] >= ((int64_t)1 << 40))
                return (int)cudaErrorInvalidValue;
            gstride[d - 1] = (cuuint64_t)strides[d - 1];
        }
    }
    if ((box[0] * 8) % 16) return (int)cudaErrorInvalidValue;
    CUtensorMap map;
    CUresult r = fn(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, (cuuint32_t)rank, const_cast<void *>(base),
                    gdim, gstride, bdim, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return (int)cudaErrorInvalidValue;
    static_assert(sizeof(CUtensorMap) == TFFT_TENSOR_MAP_BYTES, "tensor map size");
    return (int)cudaMemcpy(dev_map, &map, sizeof(map), cudaMemcpyHostToDevice);
}
