// Client program for the C++ drop-in API (include/petrichor_gb300/Petrichor.hpp).
//
// Builds a scene from a .ptscene file with the calls a Petrichor application
// makes (Vertex, Triangle, Lambert/GGX/Glass/Emission/MixMaterial,
// Scene::RegisterMaterial/AppendGeometry/AppendLight/SetMainCamera/
// SetEnvironment/SetTargetTexture/LoadRenderSetting, Environment::Load,
// Camera(pos, dir)/SetFOV/SetFocalLength/FocusTo/SetApeture, Texture2D::Load with
// Lambert::SetTexAlbedo and GGX::SetF0Texture/SetRoughnessMap/SetNormalMap and their
// strengths), renders it with Petrichor::Render and writes the Rendered texture as
// raw float32 RGB rows.
//
//   drop_in_render <scene.ptscene> <film.bin> [wavefront | aov <denoising spp>]
//   drop_in_render <scene.ptscene> <film.bin> wavefront --repeat K
//
// With --repeat the scene is built once and Petrichor::Render is called 1 + K times
// (the first call is a warm-up); the output line lists the wall seconds of the K
// timed calls. Each call does what an application's call does: flatten the scene,
// upload it, build its BVH, render, copy the film back and release the scene.
// Without "wavefront" the renderer keeps its defaults (replay mode with
// SimplePathTracing: the reference's own Render output). With "aov" the UV,
// DenoisingAlbedo and DenoisingNormal targets are set too, and the file holds the
// Rendered film followed by the three AOV films. Exit status: 0 on success, 3 when
// Render reported an error (its status code is printed).
#include <petrichor_gb300/Petrichor.hpp>
#include <petrichor_gb300.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

using namespace Petrichor;
using namespace Petrichor::Core;

namespace {

class Bytes {
public:
    explicit Bytes(const std::string& path) {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw std::runtime_error("cannot open " + path);
        m_buf.assign(std::istreambuf_iterator<char>(f), {});
    }
    void Take(void* dst, size_t n) {
        if (m_off + n > m_buf.size()) throw std::runtime_error("truncated scene file");
        std::memcpy(dst, m_buf.data() + m_off, n);
        m_off += n;
    }
    bool AtEnd() const { return m_off >= m_buf.size(); }
    template <typename T>
    T Get() {
        T v;
        Take(&v, sizeof(T));
        return v;
    }

private:
    std::vector<char> m_buf;
    size_t m_off = 0;
};

Math::Vector3f V(const float* p) { return Math::Vector3f(p[0], p[1], p[2]); }

// Everything the scene points at lives here for the lifetime of the render.
struct App {
    Scene scene;
    std::vector<Vertex> vertices;
    std::vector<Triangle> triangles;
    std::unique_ptr<Texture2D> film;
    int integrator = 0;
    int denoisingSpp = 1;
    std::unique_ptr<Texture2D> aov[3];
    std::vector<std::unique_ptr<Texture2D>> maps;  // material texture maps
};

// Writes RGB rows as the raw float container Texture2D::Load reads.
void WriteRawImage(const std::string& path, int w, int h, const float* px) {
    std::ofstream f(path, std::ios::binary);
    const uint32_t dims[2] = {(uint32_t)w, (uint32_t)h};
    f.write("PTRAWF32", 8);
    f.write(reinterpret_cast<const char*>(dims), 8);
    f.write(reinterpret_cast<const char*>(px), (std::streamsize)((size_t)w * h * 12));
    if (!f) throw std::runtime_error("cannot write " + path);
}

void BuildScene(const std::string& path, const std::string& scratch, App& app) {
    Bytes r(path);
    char magic[8];
    r.Take(magic, 8);
    if (std::memcmp(magic, "PTSCENE1", 8) != 0) throw std::runtime_error("not a .ptscene file");
    int32_t s[8];
    r.Take(s, sizeof(s));
    app.integrator = s[7];
    {  // render settings go through the JSON loader, as an application's would
        const std::string json = scratch + ".settings.json";
        std::ofstream f(json);
        f << "{\n  \"outputWidth\": " << s[0] << ",\n  \"outputHeight\": " << s[1]
          << ",\n  \"spp\": " << s[2] << ",\n  \"denoising_spp\": " << app.denoisingSpp
          << ",\n  \"maxBounces\": " << s[3]
          << ",\n  \"tileWidth\": " << s[4] << ",\n  \"tileHeight\": " << s[5]
          << ",\n  \"numThreads\": " << s[6] << "\n}\n";
        f.close();
        app.scene.LoadRenderSetting(json);
    }
    float cam[12];
    r.Take(cam, sizeof(cam));
    const uint32_t hasFocus = r.Get<uint32_t>();
    auto camera = std::make_unique<Camera>(V(cam), V(cam + 3));
    if (cam[6] > 0.0f) camera->SetFOV(cam[6]);
    else camera->SetFocalLength(cam[7]);
    if (hasFocus) camera->FocusTo(V(cam + 8));
    camera->SetApeture(cam[11]);
    app.scene.SetMainCamera(std::move(camera));

    float envf[4];
    r.Take(envf, sizeof(envf));
    const int32_t ew = r.Get<int32_t>(), eh = r.Get<int32_t>();
    (void)r.Get<uint32_t>();
    Environment env;
    env.SetBaseColor(V(envf));
    env.SetZAxisRotation(envf[3]);
    if (ew > 0 && eh > 0) {  // the texture goes through Environment::Load of an image file
        std::vector<float> px((size_t)ew * eh * 3);
        r.Take(px.data(), px.size() * 4);
        const std::string hdr = scratch + ".env.hdr";
        WriteRawImage(hdr, ew, eh, px.data());
        env.Load(hdr);
    }
    app.scene.SetEnvironment(env);

    const uint32_t M = r.Get<uint32_t>();
    std::vector<float> mf((size_t)M * 8);
    std::vector<int32_t> mi((size_t)M * 4);
    r.Take(mf.data(), mf.size() * 4);
    r.Take(mi.data(), mi.size() * 4);

    const uint32_t NV = r.Get<uint32_t>();
    std::vector<float> pos((size_t)NV * 3), nrm((size_t)NV * 3), uv((size_t)NV * 3);
    r.Take(pos.data(), pos.size() * 4);
    r.Take(nrm.data(), nrm.size() * 4);
    r.Take(uv.data(), uv.size() * 4);
    const uint32_t T = r.Get<uint32_t>();
    std::vector<int32_t> idx((size_t)T * 3), tm(T);
    std::vector<uint8_t> sh(T + (4 - T % 4) % 4);
    r.Take(idx.data(), idx.size() * 4);
    r.Take(tm.data(), tm.size() * 4);
    r.Take(sh.data(), sh.size());
    const uint32_t NL = r.Get<uint32_t>();
    std::vector<int32_t> lights(NL);
    r.Take(lights.data(), lights.size() * 4);
    if (!r.AtEnd()) {  // material texture maps, each loaded from an image file
        const uint32_t NT = r.Get<uint32_t>();
        for (uint32_t t = 0; t < NT; t++) {
            const int32_t tw = r.Get<int32_t>(), th = r.Get<int32_t>();
            std::vector<float> px((size_t)tw * th * 3);
            r.Take(px.data(), px.size() * 4);
            const std::string path = scratch + ".map" + std::to_string(t) + ".hdr";
            WriteRawImage(path, tw, th, px.data());
            app.maps.push_back(std::make_unique<Texture2D>());
            if (!app.maps.back()->Load(path, Texture2D::TextureColorType::NonColor))
                throw std::runtime_error("cannot load " + path);
        }
    }
    std::vector<uint32_t> flags(M, 0u);  // bit 0: importance sampling off
    if (!r.AtEnd()) {
        if (r.Get<uint32_t>() != M) throw std::runtime_error("material flag count");
        r.Take(flags.data(), flags.size() * 4);
    }
    // texture reference byte j of a material's int row: texture index + 1, 0 = none
    auto map = [&](int32_t refs, int j) -> const Texture2D* {
        const int r8 = (int)(((uint32_t)refs >> (8 * j)) & 0xffu);
        return r8 ? app.maps.at(r8 - 1).get() : nullptr;
    };
    std::vector<const MaterialBase*> mats(M, nullptr);
    auto name = [](uint32_t k) { return "material" + std::to_string(k); };
    for (uint32_t k = 0; k < M; k++) {  // plain materials, then mixes of them
        const float* f = &mf[(size_t)k * 8];
        std::unique_ptr<const MaterialBase> m;
        const int32_t refs = mi[(size_t)k * 4 + 3];
        switch (mi[(size_t)k * 4]) {
        case 0: {
            auto l = std::make_unique<Lambert>(V(f));
            if (map(refs, 0)) l->SetTexAlbedo(map(refs, 0));
            if (flags[k] & 1u) l->EnableImportanceSampling(false);
            m = std::move(l);
            break;
        }
        case 1: m = std::make_unique<Glass>(V(f), f[4]); break;
        case 2: m = std::make_unique<Emission>(V(f)); break;
        case 3: {
            auto g = std::make_unique<GGX>(V(f), f[3]);
            if (map(refs, 1)) g->SetF0Texture(map(refs, 1));
            if (map(refs, 2)) {
                g->SetRoughnessMap(map(refs, 2));
                g->SetRoughnessMapStrength(f[6]);
            }
            if (map(refs, 3)) {
                g->SetNormalMap(map(refs, 3));
                g->SetNormalMapStrength(f[7]);
            }
            m = std::move(g);
            break;
        }
        default: continue;
        }
        app.scene.RegisterMaterial(name(k), std::move(m));
        mats[k] = app.scene.GetMaterial(name(k));
    }
    for (uint32_t k = 0; k < M; k++) {
        const int32_t* q = &mi[(size_t)k * 4];
        if (q[0] != 4) continue;
        if (!mats.at(q[1]) || !mats.at(q[2])) throw std::runtime_error("mix of a mix");
        app.scene.RegisterMaterial(name(k),
                                   std::make_unique<MixMaterial>(mats[q[1]], mats[q[2]], mf[(size_t)k * 8 + 5]));
        mats[k] = app.scene.GetMaterial(name(k));
    }

    app.vertices.reserve(NV);
    for (uint32_t i = 0; i < NV; i++)
        app.vertices.emplace_back(V(&pos[i * 3]), V(&nrm[i * 3]), V(&uv[i * 3]));
    app.triangles.reserve(T);
    for (uint32_t t = 0; t < T; t++) {
        app.triangles.emplace_back(&app.vertices.at(idx[t * 3]), &app.vertices.at(idx[t * 3 + 1]),
                                   &app.vertices.at(idx[t * 3 + 2]),
                                   sh[t] ? ShadingTypes::Smooth : ShadingTypes::Flat);
        app.triangles.back().SetMaterial(mats.at(tm[t]));
    }
    for (const Triangle& t : app.triangles) app.scene.AppendGeometry(&t);
    for (int32_t t : lights) app.scene.AppendLight(&app.triangles.at(t));

    app.film = std::make_unique<Texture2D>(s[0], s[1]);
    app.scene.SetTargetTexture(Scene::AOVType::Rendered, app.film.get());
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <scene.ptscene> <film.bin> [wavefront | wavefront-alias | aov <spp>] [--repeat K]\n", argv[0]);
        return 2;
    }
    try {
        App app;
        const bool aov = argc > 4 && std::string(argv[3]) == "aov";
        if (aov) app.denoisingSpp = std::stoi(argv[4]);
        BuildScene(argv[1], argv[2], app);
        if (aov) {
            const Scene::AOVType::Value kinds[3] = {Scene::AOVType::UV, Scene::AOVType::DenoisingAlbedo,
                                                    Scene::AOVType::DenoisingNormal};
            for (int k = 0; k < 3; k++) {
                app.aov[k] = std::make_unique<Texture2D>(app.film->GetWidth(), app.film->GetHeight());
                app.scene.SetTargetTexture(kinds[k], app.aov[k].get());
            }
        }
        Core::Petrichor renderer;
        const std::string mode = argc > 3 ? argv[3] : "";
        if (mode == "wavefront" || mode == "wavefront-alias") renderer.SetMode(PT_MODE_WAVEFRONT);
        if (mode == "wavefront-alias") renderer.SetEnvSampling(PT_ENV_SAMPLING_ALIAS);
        renderer.SetIntegrator(app.integrator);
        float seconds = -1.0f;
        renderer.SetRenderCallback([&](const RenderingResult& r) { seconds = r.totalSec; });
        int repeat = 0;
        for (int a = 3; a + 1 < argc; a++)
            if (std::string(argv[a]) == "--repeat") repeat = std::stoi(argv[a + 1]);
        std::vector<double> calls;
        for (int k = 0; k <= repeat; k++) {
            const auto t0 = std::chrono::steady_clock::now();
            renderer.Render(app.scene);
            const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (k > 0) calls.push_back(dt);
            if (renderer.GetLastStatus() != PT_OK) break;
        }
        std::printf("{\"status\": %d, \"tiles\": [%u, %u], \"seconds\": %.6f, \"call_seconds\": [",
                    renderer.GetLastStatus(), renderer.GetNumRenderedTiles(),
                    renderer.GetNumTiles(), seconds);
        for (size_t k = 0; k < calls.size(); k++) std::printf("%s%.6f", k ? ", " : "", calls[k]);
        std::printf("]}\n");
        if (renderer.GetLastStatus() != PT_OK) {
            std::fprintf(stderr, "render failed: %s\n", renderer.GetLastError().c_str());
            return 3;
        }
        std::ofstream f(argv[2], std::ios::binary);
        for (const Texture2D* t : {app.film.get(), app.aov[0].get(), app.aov[1].get(), app.aov[2].get()})
            if (t)
                f.write(reinterpret_cast<const char*>(t->GetRawDataPtr()),
                        (std::streamsize)((size_t)t->GetWidth() * t->GetHeight() * 3 * 4));
        return f ? 0 : 1;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
