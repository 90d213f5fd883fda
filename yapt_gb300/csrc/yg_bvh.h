// Host BVH builder (see yg_bvh.cpp).
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace yg
{
// Builds the binary BVH and the leaf-ordered triangle array (layout in yg_trace.cuh).
void buildBvh(const std::vector<float3>& v0, const std::vector<float3>& v1, const std::vector<float3>& v2,
              const std::vector<uint32_t>& instance, const std::vector<uint32_t>& prim, std::vector<float4>& trisOut,
              std::vector<float4>& nodesOut);
} // namespace yg
