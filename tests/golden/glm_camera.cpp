// Camera matrices as the reference computes them, with the glm it vendors: Camera::updateProjection
// (raygun/camera.cpp:34-47: glm::perspective with depth [0,1], the Y flip), Camera::projInverse and
// viewInverse (raygun/camera.hpp:34-36: glm::inverse, Transform::toMat4 = T * R * S,
// raygun/transform.hpp:38-46), Transform::lookAt (transform.hpp:82-86: glm::quatLookAt toward the
// target with UP = +y, pch.hpp:159) and Transform::rotate (transform.hpp:74: glm::rotate of the
// quaternion).  Built and run by make_camera_golden.py against the reference's glm headers.
//
// stdin: N cases of 16 floats (fov_deg, width, height, near, far, pos xyz, mode, a, b, c, d, scale xyz);
//   mode 0: (a, b, c) = look-at target; mode 1: a = angle (radians), (b, c, d) = rotation axis.
// stdout: per case viewInverse (16, column-major), projInverse (16), rotation quaternion (w, x, y, z).
#define GLM_FORCE_DEPTH_ZERO_TO_ONE
#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>
#include <glm/gtc/quaternion.hpp>
#include <glm/gtx/quaternion.hpp>

#include <cstdio>
#include <vector>

int main() {
    std::vector<float> in;
    float x;
    while (std::fread(&x, 4, 1, stdin) == 1) in.push_back(x);
    const size_t n = in.size() / 16;
    for (size_t k = 0; k < n; ++k) {
        const float* c = &in[16 * k];
        const float aspect = c[1] / c[2];
        glm::mat4 proj = glm::perspective(glm::radians(c[0]), aspect, c[3], c[4]);
        proj[1][1] *= -1;
        const glm::mat4 projInv = glm::inverse(proj);
        const glm::vec3 pos(c[5], c[6], c[7]);
        glm::quat q = glm::identity<glm::quat>();
        if (c[8] == 0.0f) q = glm::quatLookAt(glm::normalize(glm::vec3(c[9], c[10], c[11]) - pos), glm::vec3(0.0f, 1.0f, 0.0f));
        else q = glm::rotate(q, c[9], glm::vec3(c[10], c[11], c[12]));
        const glm::mat4 id = glm::identity<glm::mat4>();
        const glm::mat4 view = glm::translate(id, pos) * glm::toMat4(q) * glm::scale(id, glm::vec3(c[13], c[14], c[15]));
        float out[36];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                out[4 * i + j] = view[i][j];
                out[16 + 4 * i + j] = projInv[i][j];
            }
        out[32] = q.w; out[33] = q.x; out[34] = q.y; out[35] = q.z;
        std::fwrite(out, 4, 36, stdout);
    }
    return 0;
}
