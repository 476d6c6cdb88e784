// Tensor-map (TMA) tile loads of lattice rows into shared memory.
//
// Every FFT pass of the step reads whole rows: density rows (N floats), the
// half spectrum's column lines (N complex = 2N floats) and so on.  A "row map"
// describes such an array to the copy engine as a 4-D tensor of 32-bit
// elements,
//     (inner, rowlen / inner, rows, batch),   inner = min(rowlen, 256),
// because one box dimension holds at most 256 elements; a box of
// (inner, rowlen / inner, tile_rows, 1) is then `tile_rows` whole rows, which
// one cp.async.bulk.tensor instruction lands densely in shared memory (at a
// 128-byte aligned address).  The map covers this GPU's own memory only (no
// multicast).  Coordinates: (0, 0, first row, lattice of the batch); the
// innermost coordinate is always 0, so the 16-byte alignment rule of the
// innermost coordinate holds trivially.
#pragma once

#include <cuda.h>
#include <stdint.h>

#include "bulk_copy.cuh"

namespace cpm {
namespace tma {

// Rows [row, row + box_rows) of lattice `batch` into `dst` (shared memory,
// 128-byte aligned); completion counts down the transaction bytes of `bar`.
__device__ __forceinline__ void load_rows(void* dst, const CUtensorMap* map, int row, int batch, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(bulk::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(0), "r"(row), "r"(batch), "r"(bulk::smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Thread 0 arms `bar` for `bytes` and issues the load; every thread of the CTA
// then waits (bounded).  Returns false in a thread whose wait timed out.
__device__ __forceinline__ bool load_rows_sync(void* dst, const CUtensorMap* map, int row, int batch, uint32_t bytes,
                                               uint64_t* bar, uint32_t parity) {
    if (threadIdx.x == 0) {
        bulk::arrive_expect_tx(bar, bytes);
        load_rows(dst, map, row, batch, bar);
    }
    return bulk::wait(bar, parity);
}

}  // namespace tma
}  // namespace cpm
