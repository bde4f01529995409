// The reference's own glm (its vendored copy, glm 0.9.8.5) for the math the
// oracle restates. TEST INFRASTRUCTURE ONLY: compiled from the reference tree
// by oracle/build_ref.py into oracle/_ref/ (a no-op where the tree is
// absent); tests/test_oracle_glm.py compares the oracle's conventions with it.
//
//   glmref_vecmath: glm's dot, cross, length, normalize, mix and mat4 * vec4
//     over n inputs (the shaders' GLSL builtins as glm evaluates them);
//   glmref_fps_camera: the reference's camera, built as Core/FpsCamera.cpp
//     builds it (UpdateOnMouseMovement :59-72 for the front vector,
//     RecalculateViewMatrix / RecalculateProjectionMatrix for lookAt and
//     perspective) and inverted as Core/Pipeline.cpp:1823-1824 does.
#include <cmath>
#include <cstring>

#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>

extern "C" {

// op 0: dot(a, b); 1: cross(a, b); 2: length(a); 3: normalize(a);
// 4: mix(a.x, b.x, c.x) (scalar); 5: mat4(a) * vec4(b) (a: 16 floats column-major
// per item, b: 4 floats). a, b, c and out hold n items of 3 floats (16 / 4 / 4 for op 5).
void glmref_vecmath(int op, const float* a, const float* b, const float* c, float* out, int n) {
    for (int k = 0; k < n; k++) {
        if (op == 5) {
            glm::mat4 m;
            std::memcpy(&m[0][0], a + 16 * k, 64);
            const glm::vec4 v(b[4 * k], b[4 * k + 1], b[4 * k + 2], b[4 * k + 3]);
            const glm::vec4 r = m * v;
            for (int i = 0; i < 4; i++) out[4 * k + i] = r[i];
            continue;
        }
        const glm::vec3 x(a[3 * k], a[3 * k + 1], a[3 * k + 2]);
        const glm::vec3 y(b[3 * k], b[3 * k + 1], b[3 * k + 2]);
        glm::vec3 r(0.0f);
        switch (op) {
            case 0: r.x = glm::dot(x, y); break;
            case 1: r = glm::cross(x, y); break;
            case 2: r.x = glm::length(x); break;
            case 3: r = glm::normalize(x); break;
            case 4: r.x = glm::mix(x.x, y.x, c[3 * k]); break;
            default: break;
        }
        out[3 * k] = r.x;
        out[3 * k + 1] = r.y;
        out[3 * k + 2] = r.z;
    }
}

// The camera of a player at `pos` looking along (yaw, pitch) in degrees.
void glmref_fps_camera(const float* pos, float yaw, float pitch, float fov, float aspect, float znear, float zfar,
                       float* view, float* proj, float* inv_view, float* inv_proj) {
    glm::vec3 front;
    front.x = cos(glm::radians(pitch)) * cos(glm::radians(yaw));
    front.y = sin(glm::radians(pitch));
    front.z = cos(glm::radians(pitch)) * sin(glm::radians(yaw));
    const glm::vec3 position(pos[0], pos[1], pos[2]);
    const glm::mat4 v = glm::lookAt(position, front + position, glm::vec3(0.0f, 1.0f, 0.0f));
    const glm::mat4 p = glm::perspective(glm::radians(fov), aspect, znear, zfar);
    const glm::mat4 iv = glm::inverse(v), ip = glm::inverse(p);
    std::memcpy(view, &v[0][0], 64);
    std::memcpy(proj, &p[0][0], 64);
    std::memcpy(inv_view, &iv[0][0], 64);
    std::memcpy(inv_proj, &ip[0][0], 64);
}

}  // extern "C"
