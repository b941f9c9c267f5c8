// Stand-ins for Core/SceneLoader.cpp (nlohmann-json) and Core/Geometry/Mesh.cpp
// (Assimp), whose libraries are not available here. The oracle harness builds
// scenes through the C++ API instead, so both loaders only report an error.
// Test oracle build only.
#include "Core/Geometry/Mesh.h"
#include "Core/SceneLoader.h"

#include <cstdio>

namespace Petrichor {
namespace Core {

void SceneLoaderJson::Load(const std::filesystem::path& path, Scene&) {
    std::fprintf(stderr, "[oracle] SceneLoaderJson unavailable in this build: %s\n",
                 path.string().c_str());
}

void Mesh::Load(const std::filesystem::path& path, const MaterialBase*, ShadingTypes) {
    std::fprintf(stderr, "[oracle] Mesh::Load unavailable in this build: %s\n",
                 path.string().c_str());
}

}  // namespace Core
}  // namespace Petrichor
