// Camera matrices of the C++ facade (include/rg/raygun.hpp) for the cases of
// tests/golden/camera_glm.npz, in the same binary layout as tests/golden/glm_camera.cpp:
// stdin N x 16 floats (fov_deg, width, height, near, far, pos xyz, mode, a, b, c, d, scale xyz),
// stdout N x 36 floats (viewInverse, projInverse, rotation w x y z).
#include <cstdio>
#include <vector>

#include "rg/raygun.hpp"

int main() {
    std::vector<float> in;
    float x;
    while (std::fread(&x, 4, 1, stdin) == 1) in.push_back(x);
    const size_t n = in.size() / 16;
    for (size_t k = 0; k < n; ++k) {
        const float* c = &in[16 * k];
        rg::Camera cam;
        cam.fovDegrees = c[0];
        cam.zNear = c[3];
        cam.zFar = c[4];
        rg::Transform t;
        t.position = rg::vec3(c[5], c[6], c[7]);
        if (c[8] == 0.0f) t.lookAt(rg::vec3(c[9], c[10], c[11]));
        else t.rotate(c[9], rg::vec3(c[10], c[11], c[12]));
        t.scaling = rg::vec3(c[13], c[14], c[15]);
        cam.setTransform(t);
        cam.updateProjection((uint32_t)c[1], (uint32_t)c[2]);
        const rg::mat4 v = cam.viewInverse(), p = cam.projInverse();
        float out[36];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                out[4 * i + j] = v.m[i][j];
                out[16 + 4 * i + j] = p.m[i][j];
            }
        out[32] = t.rotation.w; out[33] = t.rotation.x; out[34] = t.rotation.y; out[35] = t.rotation.z;
        std::fwrite(out, 4, 36, stdout);
    }
    return 0;
}
