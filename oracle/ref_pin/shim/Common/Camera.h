// Stand-in for glim::Camera (only its declarations are needed by the pin build).
#pragma once
#include <glm/glm.hpp>
namespace glim {
struct Camera {
    glm::dvec3 ViewPosition;
    glm::mat4 GetProjMatrix() const { return glm::mat4(); }
    glm::mat4 GetViewMatrix(bool) const { return glm::mat4(); }
};
}  // namespace glim
