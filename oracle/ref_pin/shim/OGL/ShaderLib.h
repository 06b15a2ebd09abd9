// Stand-in for ogl::ShaderLib (shader loading is never executed by the pin driver).
#pragma once
#include <memory>
#include <string_view>
#include <vector>
#include "QuickGL.h"
namespace ogl {
struct ShaderLoadParams {
    struct PrepDef {
        std::string_view Name, Value;
    };
};
struct ShaderLib {
    std::shared_ptr<Shader> LoadComp(std::string_view, const std::vector<ShaderLoadParams::PrepDef>& = {}) {
        return std::make_shared<Shader>();
    }
    std::shared_ptr<Shader> LoadFrag(std::string_view) { return std::make_shared<Shader>(); }
};
}  // namespace ogl
