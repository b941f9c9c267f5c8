// Client program for the file loaders of the C++ API: loads a render-settings file and
// a JSON scene file (with OBJ assets and a Radiance .hdr environment) exactly as the
// reference application does (Scene::LoadRenderSetting, Scene::LoadAssets), then
//
//   load_scene dump   <settings> <scene.json> <out.txt>  writes what was loaded as text
//   load_scene render <settings> <scene.json> <out.bin>  renders (replay) and writes the film
//   load_scene save   <in.hdr> <out.png> <out.hdr>       loads an image and saves it both ways
//   load_scene tex    <in> <out.bin> color|noncolor        loads an image (Texture2D::Load) and
//                                                          writes int32 width, height, RGB floats
//   load_scene sample <in> <out.txt> <u v>...              GetPixelByUV (bilinear, then point)
//
// The text dump holds one record per line with floats as C99 hex literals, so the
// test reads back exact values.
#include <petrichor_gb300/Petrichor.hpp>
#include <petrichor_gb300.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <string>
#include <utility>
#include <vector>

using namespace Petrichor;
using namespace Petrichor::Core;

namespace {

void Put(FILE* f, const Math::Vector3f& v) { std::fprintf(f, " %a %a %a", v.x, v.y, v.z); }

int Dump(const Scene& scene, const char* out) {
    FILE* f = std::fopen(out, "w");
    if (!f) return 1;
    const RenderSetting& rs = scene.GetRenderSetting();
    std::fprintf(f, "settings %d %d %d %d %d %d %d %d\n", rs.outputWidth, rs.outputHeight,
                 rs.numSamplesPerPixel, rs.numSppForDenoising, rs.numMaxBounces, rs.tileWidth,
                 rs.tileHeight, rs.numThreads);
    const Camera* c = scene.GetMainCamera();
    std::fprintf(f, "camera");
    Put(f, c->Position());
    Put(f, c->Forward());
    Put(f, c->Right());
    Put(f, c->Up());
    std::fprintf(f, " %a %a %a\n", c->GetHPerf(), c->GetFocusDist(), c->GetApeture());
    const Environment& env = scene.GetEnvironment();
    std::fprintf(f, "env");
    Put(f, env.GetBaseColor());
    const Texture2D* t = env.GetTexture();
    std::fprintf(f, " %d %d\n", t ? t->GetWidth() : 0, t ? t->GetHeight() : 0);
    if (t)
        for (int j = 0; j < t->GetHeight(); j++)
            for (int i = 0; i < t->GetWidth(); i++) {
                std::fprintf(f, "texel");
                Put(f, t->GetPixel(i, j));
                std::fprintf(f, "\n");
            }
    std::map<const MaterialBase*, int> ids;
    auto id = [&](const MaterialBase* m) {
        auto it = ids.find(m);
        if (it != ids.end()) return it->second;
        const int k = (int)ids.size();
        ids[m] = k;
        std::fprintf(f, "material %d %d", k, m ? (int)m->GetMaterialType() : -1);
        // texture maps: "map <material> <slot> <width> <height> <strength> <texels...>"
        std::vector<std::pair<int, const Texture2D*>> maps;
        float strength = 1.0f;
        if (m && m->GetMaterialType() == MaterialTypes::Lambert) {
            Put(f, static_cast<const Lambert*>(m)->GetKd());
            maps.push_back({0, static_cast<const Lambert*>(m)->GetTexAlbedo()});
        }
        if (m && m->GetMaterialType() == MaterialTypes::Glossy) {
            const auto* g = static_cast<const GGX*>(m);
            Put(f, g->GetReflectance());
            std::fprintf(f, " %a", g->GetRoughness());
            maps.push_back({1, g->GetF0Texture()});
            maps.push_back({2, g->GetRoughnessMap()});
            strength = g->GetRoughnessMapStrength();
        }
        if (m && m->GetMaterialType() == MaterialTypes::Glass) {
            Put(f, static_cast<const Glass*>(m)->GetColor());
            std::fprintf(f, " %a", static_cast<const Glass*>(m)->GetIOR());
        }
        if (m && m->GetMaterialType() == MaterialTypes::Mix) {
            const auto* x = static_cast<const MixMaterial*>(m);
            std::fprintf(f, " %a", x->GetMix());
        }
        std::fprintf(f, "\n");
        for (const auto& [slot, t] : maps) {
            if (!t) continue;
            std::fprintf(f, "map %d %d %d %d %a", k, slot, t->GetWidth(), t->GetHeight(), strength);
            for (int j = 0; j < t->GetHeight(); j++)
                for (int i = 0; i < t->GetWidth(); i++) Put(f, t->GetPixel(i, j));
            std::fprintf(f, "\n");
        }
        return k;
    };
    for (const GeometryBase* g : scene.GetGeometries()) {
        const auto* tri = static_cast<const Triangle*>(g);
        const int m = id(tri->GetMaterialPointer());
        if (tri->GetMaterialPointer() && tri->GetMaterialPointer()->GetMaterialType() == MaterialTypes::Mix) {
            const auto* x = static_cast<const MixMaterial*>(tri->GetMaterialPointer());
            std::fprintf(f, "mixof %d %d %d\n", m, id(x->GetMat0()), id(x->GetMat1()));
        }
        std::fprintf(f, "tri %d %d", m, tri->GetShadingType() == ShadingTypes::Smooth ? 1 : 0);
        for (const Vertex* v : tri->GetVertices()) {
            Put(f, v->pos);
            Put(f, v->normal);
            Put(f, v->uv);
        }
        std::fprintf(f, "\n");
    }
    std::fclose(f);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s dump|render <settings> <scene.json> <out> | save <in.hdr> <out.png> <out.hdr>\n",
                     argv[0]);
        return 2;
    }
    const std::string mode = argv[1];
    if (mode == "sample") {
        Texture2D tex;
        if (!tex.Load(argv[2], Texture2D::TextureColorType::NonColor)) return 4;
        FILE* f = std::fopen(argv[3], "w");
        if (!f) return 1;
        for (int k = 4; k + 1 < argc; k += 2) {
            const float u = std::strtof(argv[k], nullptr), v = std::strtof(argv[k + 1], nullptr);
            Put(f, tex.GetPixelByUV(u, v));
            Put(f, tex.GetPixelByUV(u, v, Texture2D::InterplationTypes::Point));
            std::fprintf(f, "\n");
        }
        std::fclose(f);
        return 0;
    }
    if (mode == "tex") {
        Texture2D tex;
        const bool color = std::string(argv[4]) == "color";
        if (!tex.Load(argv[2], color ? Texture2D::TextureColorType::Color
                                     : Texture2D::TextureColorType::NonColor))
            return 4;
        std::ofstream o(argv[3], std::ios::binary);
        const int32_t dims[2] = {tex.GetWidth(), tex.GetHeight()};
        o.write(reinterpret_cast<const char*>(dims), 8);
        o.write(reinterpret_cast<const char*>(tex.GetRawDataPtr()),
                (std::streamsize)((size_t)dims[0] * dims[1] * 3 * 4));
        return o ? 0 : 1;
    }
    if (mode == "save") {
        Texture2D tex;
        if (!tex.Load(argv[2])) return 4;
        tex.Save(argv[3]);
        tex.Save(argv[4]);
        return 0;
    }
    Scene scene;
    scene.LoadRenderSetting(argv[2]);
    scene.LoadAssets(argv[3]);
    if (mode == "dump") return Dump(scene, argv[4]);
    const RenderSetting& rs = scene.GetRenderSetting();
    Texture2D film(rs.outputWidth, rs.outputHeight);
    scene.SetTargetTexture(Scene::AOVType::Rendered, &film);
    Core::Petrichor renderer;
    renderer.Render(scene);
    if (renderer.GetLastStatus() != PT_OK) {
        std::fprintf(stderr, "render failed: %s\n", renderer.GetLastError().c_str());
        return 3;
    }
    std::ofstream o(argv[4], std::ios::binary);
    o.write(reinterpret_cast<const char*>(film.GetRawDataPtr()),
            (std::streamsize)((size_t)film.GetWidth() * film.GetHeight() * 3 * 4));
    return o ? 0 : 1;
}
