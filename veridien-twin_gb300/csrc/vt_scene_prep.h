// Scene preparation shared between the host restatement (vt_scene_prep.cpp) and the device versions
// (vt_scene_gpu.cu): results handed out through vt_mesh_out, released by vt_mesh_free.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/vtwin.h"

namespace vt {
// moves the arrays into a library-owned mesh (out->handle) that vt_mesh_free releases
vt_status mesh_hand_out(std::vector<double>&& P, std::vector<double>&& N, std::vector<uint32_t>&& I, vt_mesh_out* out);
}  // namespace vt
