// capi_internal.h -- helpers shared by capi.cu and sim.cu.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "amr_gb300.h"
#include "kernels.h"
#include "octree.h"

namespace amr {

int cuda_status(cudaError_t e);
bool config_supported(const amr_config* c);
bool bssn_fused_supported(const amr_config* c);
cudaError_t launch_stencil(const amr_config& c, int kind, const StencilArgs& a, uint32_t grid, cudaStream_t st);
uint32_t stencil_grid(const amr_config& c, int kind, uint32_t n_items);
int* device_error_flag();
int take_device_error(int* flag);
int octree_state_impl(const Octree& t, uint32_t* positions, int32_t* parent, int32_t* children, uint64_t* boundaries,
                      uint32_t* lifetime, uint32_t* scalars);

}  // namespace amr
