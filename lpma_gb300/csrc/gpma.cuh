// GPMA mode (LPMA_FLAG_GPMA): the flat packed memory array of the
// reference's gpma.cuh as a configuration of the engine's update pipeline.
// Definitions in gpma.cu; the C ABI in abi.cu dispatches here for handles
// created with the flag.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "lpma.h"

namespace lpma {

constexpr uint64_t GPMA_KEY_MAX = 0xFFFFFFFFFFFFFFFEull;  // KEY_MAX guards, gpma.cuh:30, 818-823

struct GpmaState;

// stream-ordered allocation from the engine's memory pool (abi.cu)
cudaError_t pool_alloc(void **p, size_t bytes, cudaStream_t s);
// reserved bytes of the current device's update memory pool
uint64_t pool_reserved_bytes();

lpma_status_t gpma_create(uint32_t num_vertices, double density_lower, cudaStream_t s, GpmaState **out);
void gpma_destroy(GpmaState *g);
lpma_status_t gpma_update(GpmaState *g, const uint64_t *ins, const uint8_t *ins_vals, size_t n_ins, const uint64_t *del,
                          size_t n_del, cudaStream_t s, LpmaStats *out);
lpma_status_t gpma_geometry(const GpmaState *g, uint64_t *size, uint32_t *seg, uint32_t *height, uint64_t *num_items);
lpma_status_t gpma_view(GpmaState *g, const uint32_t **row_offset, const uint64_t **keys, const uint8_t **vals);
lpma_status_t gpma_export_layout(GpmaState *g, uint64_t *h_keys, uint8_t *h_vals, size_t cap_slots,
                                 uint32_t *row_offset, size_t cap_rows, cudaStream_t s);
lpma_status_t gpma_export_sorted(GpmaState *g, uint64_t *h_keys, uint8_t *h_vals, size_t cap, size_t *n_out,
                                 cudaStream_t s);
uint64_t gpma_memory_bytes(const GpmaState *g);

}  // namespace lpma
