// pipeline.cuh — internal entry points shared by the recognition pipeline.
#pragma once
#include "icp.cuh"

namespace rtr {

// Scratch need of rtr_recognize for a scene of n points and a model.
size_t recognize_scratch_bytes(int n_scene, int n_model_vox, int n_model_kp, const rtr_recog_params* p,
                               bool learned = false);

}  // namespace rtr
