// Host-side helpers (pixel table, camera, synthetic scenes).
#pragma once

#include <cstdint>
#include <vector>

namespace wfpt {

void pixel_table(int width, int height, int32_t* idx_to_pix, int32_t* pix_to_idx);
bool camera_screen_to_world(const float pos[3], const float rot_deg[3], float fov_deg, float aspect, float znear,
                            float zfar, float out[16]);
bool generate_scene(int kind, uint64_t seed, uint32_t ntri, std::vector<float>& pos, std::vector<float>& nrm,
                    std::vector<uint32_t>& idx);

}  // namespace wfpt
