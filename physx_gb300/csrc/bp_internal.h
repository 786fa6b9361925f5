// Broadphase hooks used inside libgbpx by the large-scene step (scene.cu):
// the ABP instance of gbpx_bp_* driven from device-resident bounds, with its
// active pair set read in place.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbpx
{
namespace bpi
{
// Handles [0, n), created earlier through gbpx_bp_update, take new bounds from
// device memory (6 floats per handle: min xyz, max xyz; distance 0) and are
// marked updated; the frame runs to completion on the broadphase's stream.
int updateFromDevice(void* bp, const float* dBounds, uint32_t n);
// Active pair set after the last frame: device array of keys (id0 << 32 | id1),
// id0 < id1, sorted ascending; valid until the next update.
const unsigned long long* activePairs(void* bp, uint32_t* count);
cudaStream_t stream(void* bp);
} // namespace bpi
} // namespace gbpx
