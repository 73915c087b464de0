// pipeline.cuh — internal entry points shared by the recognition pipeline.
#pragma once
#include "icp.cuh"

namespace rtr {

// Scratch need of rtr_recognize for a scene of n points.
size_t recognize_scratch_bytes(int n_scene, const rtr_recog_params* p, bool learned);

}  // namespace rtr
