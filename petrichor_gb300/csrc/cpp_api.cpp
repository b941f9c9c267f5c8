// The C++ scene/renderer API (include/petrichor_gb300/Petrichor.hpp) over the C ABI.
//
// Camera arithmetic restates the reference's (Core/Camera.cpp:23-44), so the
// derived state handed to the kernels is the same float by float; built with
// -ffp-contract=off like the rest of the host code.
#include "petrichor_gb300/Petrichor.hpp"

#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>

#include "petrichor_gb300.h"

namespace Petrichor {
namespace Math {

float Vector3f::Length() const { return (float)std::sqrt((double)Dot(*this, *this)); }
Vector3f Vector3f::Normalized() const { return *this / Length(); }

}  // namespace Math

namespace Core {

namespace {
constexpr float kPi = 3.14159265358979f;

std::string Slurp(const std::filesystem::path& path, bool* ok) {
    std::ifstream f(path, std::ios::in | std::ios::binary);
    *ok = !f.fail();
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// "key": <int> pairs of a flat JSON object.
std::map<std::string, long> JsonInts(const std::string& s) {
    std::map<std::string, long> out;
    size_t i = 0;
    while ((i = s.find('"', i)) != std::string::npos) {
        const size_t j = s.find('"', i + 1);
        if (j == std::string::npos) break;
        const std::string key = s.substr(i + 1, j - i - 1);
        size_t k = j + 1;
        while (k < s.size() && std::isspace((unsigned char)s[k])) k++;
        if (k < s.size() && s[k] == ':') {
            k++;
            while (k < s.size() && std::isspace((unsigned char)s[k])) k++;
            size_t e = k;
            if (e < s.size() && (s[e] == '-' || s[e] == '+')) e++;
            while (e < s.size() && std::isdigit((unsigned char)s[e])) e++;
            if (e > k) out[key] = std::stol(s.substr(k, e - k));
            i = e;
        } else {
            i = j + 1;
        }
    }
    return out;
}

// "[table]" headers and "key = <int>" lines, reported as "table.key".
std::map<std::string, long> TomlInts(const std::string& s) {
    std::map<std::string, long> out;
    std::istringstream in(s);
    std::string line, table;
    while (std::getline(in, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        const size_t a = line.find_first_not_of(" \t\r");
        if (a == std::string::npos) continue;
        line = line.substr(a);
        if (line[0] == '[') {
            const size_t b = line.find(']');
            table = line.substr(1, b == std::string::npos ? std::string::npos : b - 1);
            continue;
        }
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string key = line.substr(0, eq);
        key = key.substr(0, key.find_last_not_of(" \t") + 1);
        const std::string val = line.substr(eq + 1);
        const size_t v0 = val.find_first_not_of(" \t");
        if (v0 == std::string::npos) continue;
        try {
            out[table.empty() ? key : table + "." + key] = std::stol(val.substr(v0));
        } catch (...) {
        }
    }
    return out;
}

void Read(int* dst, const std::map<std::string, long>& kv, const char* key) {
    const auto it = kv.find(key);
    if (it != kv.end()) *dst = (int)it->second;
    else std::cerr << "RenderSetting: key is not found. [" << key << "]\n";
}
}  // namespace

// ---------------------------------------------------------------- Texture2D
Texture2D::Texture2D(int width, int height) : m_width(width), m_height(height) { Clear(); }

void Texture2D::Clear(const Color3f& c) {
    m_pixels.assign((size_t)std::max(m_width, 0) * std::max(m_height, 0) * 3, 0.0f);
    for (size_t i = 0; i < m_pixels.size(); i += 3) {
        m_pixels[i] = c.x;
        m_pixels[i + 1] = c.y;
        m_pixels[i + 2] = c.z;
    }
}

Color3f Texture2D::GetPixel(float x, float y, InterplationTypes type) const {  // Texture2D.cpp:273-326
    if (type == InterplationTypes::Point) return GetPixel(static_cast<int>(x), static_cast<int>(y));
    int ix0 = static_cast<int>(x), ix1 = static_cast<int>(x + 1.0f);
    int iy0 = static_cast<int>(y), iy1 = static_cast<int>(y + 1.0f);
    const float wx0 = x - ix0, wy0 = y - iy0, wx1 = ix1 - x, wy1 = iy1 - y;
    ix0 = std::clamp(ix0, 0, GetWidth() - 1);
    ix1 = std::clamp(ix1, 0, GetWidth() - 1);
    iy0 = std::clamp(iy0, 0, GetHeight() - 1);
    iy1 = std::clamp(iy1, 0, GetHeight() - 1);
    const Color3f top = wx1 * GetPixel(ix0, iy0) + wx0 * GetPixel(ix1, iy0);
    const Color3f bottom = wx1 * GetPixel(ix0, iy1) + wx0 * GetPixel(ix1, iy1);
    return wy1 * top + wy0 * bottom;
}

Color3f Texture2D::GetPixelByUV(float u, float v, InterplationTypes type) const {  // Texture2D.cpp:328-335
    u = u - 1.0f * std::floor(u / 1.0f);  // Math::Mod (MathUtils.h:32-36)
    v = v - 1.0f * std::floor(v / 1.0f);
    return GetPixel(u * m_width, v * m_height, type);
}

Color3f Texture2D::GetPixel(int i, int j) const {  // Texture2D.cpp:260-271
    if (!IsValid()) return Color3f(1.0f, 0.0f, 1.0f);
    const float* p = &m_pixels[((size_t)m_width * j + i) * 3];
    return Color3f(p[0], p[1], p[2]);
}

void Texture2D::SetPixel(int i, int j, const Color3f& c) {
    float* p = &m_pixels[((size_t)m_width * j + i) * 3];
    p[0] = c.x;
    p[1] = c.y;
    p[2] = c.z;
}

// ---------------------------------------------------------------- Environment
void Environment::Load(const std::filesystem::path& path) {
    auto t = std::make_shared<Texture2D>();
    if (t->Load(path)) m_tex = t;
}

void Environment::SetTexture(const Texture2D& texture) {
    m_tex = std::make_shared<Texture2D>(texture);
    m_tex->SetLoaded(true);
}

// ---------------------------------------------------------------- Camera (Camera.cpp:23-44)
Camera::Camera(const Math::Vector3f& pos, const Math::Vector3f& dir) : m_pos(pos) { SetViewDir(dir); }
void Camera::SetFocalLength(float focalLength) { m_hPerf = m_sensorHeight / focalLength; }
void Camera::FocusTo(const Math::Vector3f& target) { m_focusDist = (target - m_pos).Length(); }
void Camera::SetFOV(float fov) { m_hPerf = (float)(2.0f * std::tan((double)(0.5f * fov))); }
void Camera::SetViewDir(const Math::Vector3f& dir) {
    m_forward = dir.Normalized();
    m_right = Math::Cross(m_forward, Math::Vector3f::UnitZ());
    m_up = Math::Cross(m_right, m_forward);
}
void Camera::LookAt(const Math::Vector3f& target) { SetViewDir(target - m_pos); }
float Camera::GetFOV() const { return (float)(2.0f * std::atan((double)(0.5f * m_sensorHeight / m_focusDist))); }
float Camera::GetLensArea() const { return kPi * (0.5f * m_apeture) * (0.5f * m_apeture); }

// ---------------------------------------------------------------- Scene
void Scene::LoadRenderSetting(const std::filesystem::path& path) {
    bool ok = false;
    const std::string text = Slurp(path, &ok);
    if (!ok) {
        std::cerr << "Failed to read the render setting file. [" << path.string() << "]\n";
        return;
    }
    RenderSetting rs;
    if (path.extension() == ".toml") {  // RenderSettingLoader.cpp:105-124
        const auto kv = TomlInts(text);
        Read(&rs.outputWidth, kv, "settings.render_width");
        Read(&rs.outputHeight, kv, "settings.render_height");
        Read(&rs.numSamplesPerPixel, kv, "settings.spp");
        Read(&rs.numMaxBounces, kv, "settings.maxBounces");
        Read(&rs.tileWidth, kv, "settings.tile_width");
        Read(&rs.tileHeight, kv, "settings.tile_height");
        Read(&rs.numThreads, kv, "settings.num_threads");
    } else {  // RenderSettingLoader.cpp:49-64
        const auto kv = JsonInts(text);
        Read(&rs.outputWidth, kv, "outputWidth");
        Read(&rs.outputHeight, kv, "outputHeight");
        Read(&rs.numSamplesPerPixel, kv, "spp");
        Read(&rs.numSppForDenoising, kv, "denoising_spp");
        Read(&rs.numMaxBounces, kv, "maxBounces");
        Read(&rs.tileWidth, kv, "tileWidth");
        Read(&rs.tileHeight, kv, "tileHeight");
        Read(&rs.numThreads, kv, "numThreads");
    }
    m_renderSetting = rs;
}

// ---------------------------------------------------------------- Petrichor::Render
IntelOpenImageDenoiser::IntelOpenImageDenoiser() = default;
IntelOpenImageDenoiser::~IntelOpenImageDenoiser() {
    if (m_ctx) pt_context_destroy(m_ctx);
}

Texture2D IntelOpenImageDenoiser::Run(const Texture2D& color, const Texture2D* albedo,
                                      const Texture2D* normal, bool isHDR) {
    Texture2D out(color.GetWidth(), color.GetHeight());
    auto error = [&](const std::string& msg) {
        std::cerr << "[Error] " << msg << "\n";
        return out;
    };
    for (const Texture2D* t : {albedo, normal})
        if (t && (t->GetWidth() != color.GetWidth() || t->GetHeight() != color.GetHeight()))
            return error("denoiser guide image size differs from the colour image");
    if (!m_ctx) {
        const int rc = pt_context_create(0, 0, &m_ctx);
        if (rc != PT_OK) {
            m_ctx = nullptr;
            return error(std::string("no GPU context: ") + pt_status_string(rc));
        }
    }
    const int rc = pt_denoise(m_ctx, color.GetWidth(), color.GetHeight(), color.GetRawDataPtr(),
                              albedo ? albedo->GetRawDataPtr() : nullptr,
                              normal ? normal->GetRawDataPtr() : nullptr, isHDR ? 1 : 0,
                              out.GetRawDataPtr());
    if (rc != PT_OK) return error(pt_last_error(m_ctx));
    return out;
}

Texture2D IntelOpenImageDenoiser::Denoise(const Texture2D& color, bool isHDR) {
    return Run(color, nullptr, nullptr, isHDR);
}

Texture2D IntelOpenImageDenoiser::Denoise(const Texture2D& color, const Texture2D& albedo,
                                          const Texture2D& normal, bool isHDR) {
    return Run(color, &albedo, &normal, isHDR);
}

Petrichor::Petrichor() = default;
Petrichor::~Petrichor() {
    if (m_ctx) pt_context_destroy(m_ctx);
}

uint32_t Petrichor::GetNumRenderedTiles() const {
    uint32_t d = 0, t = 0;
    if (m_ctx) pt_get_progress(m_ctx, &d, &t);
    return d;
}

uint32_t Petrichor::GetNumTiles() const {
    uint32_t d = 0, t = 0;
    if (m_ctx) pt_get_progress(m_ctx, &d, &t);
    return t;
}

void Petrichor::Render(const Scene& scene) {
    const auto t0 = std::chrono::steady_clock::now();
    auto fail = [&](int status, const std::string& msg) {
        m_lastStatus = status;
        m_lastError = msg;
        std::cerr << "[Error] " << msg << "\n";
    };
    m_lastStatus = PT_OK;
    m_lastError.clear();
    Texture2D* target = scene.GetTargetTexture(Scene::AOVType::Rendered);
    bool anyTarget = target != nullptr;
    for (int a = Scene::AOVType::UV; a < Scene::AOVType::NumAOVTypes; a++)
        anyTarget = anyTarget || scene.GetTargetTexture((Scene::AOVType::Value)a) != nullptr;
    if (!anyTarget) return fail(PT_ERR_INVALID_ARG, "Target texture has not been set.");
    const Camera* cam = scene.GetMainCamera();
    if (!cam) return fail(PT_ERR_INVALID_ARG, "Main camera is not found.");
    if (!m_ctx) {
        const int rc = pt_context_create(0, 0, &m_ctx);
        if (rc != PT_OK) return fail(rc, std::string("no GPU context: ") + pt_status_string(rc));
    }

    // flatten what the render reads (Scene.h:95-173)
    std::vector<float> pos, nrm, uv;
    std::vector<int32_t> idx, triMat, lights;
    std::vector<uint8_t> shading;
    std::vector<pt_material> mats;
    std::vector<pt_texture> textures;
    std::unordered_map<const Texture2D*, int32_t> texIndex;
    std::string texError;
    // texture reference of a material map: 1 + index, 0 for none
    auto addTexture = [&](const Texture2D* t) -> int32_t {
        if (!t) return 0;
        auto it = texIndex.find(t);
        if (it != texIndex.end()) return it->second;
        if (t->GetWidth() <= 0 || t->GetHeight() <= 0) texError = "material texture is empty";
        textures.push_back(pt_texture{t->GetWidth(), t->GetHeight(), t->GetRawDataPtr()});
        return texIndex[t] = (int32_t)textures.size();
    };
    std::unordered_map<const MaterialBase*, int32_t> matIndex;
    std::function<int32_t(const MaterialBase*)> addMaterial = [&](const MaterialBase* m) -> int32_t {
        auto it = matIndex.find(m);
        if (it != matIndex.end()) return it->second;
        pt_material pm{};
        switch (m->GetMaterialType()) {
        case MaterialTypes::Lambert: {
            const auto* l = static_cast<const Lambert*>(m);
            pm.kind = PT_MAT_LAMBERT;
            pm.color[0] = l->GetKd().x, pm.color[1] = l->GetKd().y, pm.color[2] = l->GetKd().z;
            pm.tex_albedo = addTexture(l->GetTexAlbedo());
            pm.uniform_sampling = l->IsImportanceSamplingEnabled() ? 0 : 1;
            break;
        }
        case MaterialTypes::Glossy: {
            const auto* g = static_cast<const GGX*>(m);
            pm.kind = PT_MAT_GLOSSY;
            const Color3f& c = g->GetReflectance();
            pm.color[0] = c.x, pm.color[1] = c.y, pm.color[2] = c.z;
            pm.roughness = g->GetRoughness();
            pm.tex_f0 = addTexture(g->GetF0Texture());
            pm.tex_roughness = addTexture(g->GetRoughnessMap());
            pm.tex_normal = addTexture(g->GetNormalMap());
            pm.roughness_strength = g->GetRoughnessMapStrength();
            pm.normal_strength = g->GetNormalMapStrength();
            break;
        }
        case MaterialTypes::Glass: {
            const auto* g = static_cast<const Glass*>(m);
            pm.kind = PT_MAT_GLASS;
            const Color3f& c = g->GetColor();
            pm.color[0] = c.x, pm.color[1] = c.y, pm.color[2] = c.z;
            pm.ior = g->GetIOR();
            break;
        }
        case MaterialTypes::Emission: {
            const Color3f& c = static_cast<const Emission*>(m)->GetLightColor();
            pm.kind = PT_MAT_EMISSION;
            pm.color[0] = c.x, pm.color[1] = c.y, pm.color[2] = c.z;
            break;
        }
        case MaterialTypes::Mix: {
            const auto* x = static_cast<const MixMaterial*>(m);
            pm.kind = PT_MAT_MIX;
            pm.mat0 = addMaterial(x->GetMat0());
            pm.mat1 = addMaterial(x->GetMat1());
            pm.mix = x->GetMix();
            break;
        }
        }
        mats.push_back(pm);
        return matIndex[m] = (int32_t)mats.size() - 1;
    };
    // every triangle gets its own three corner vertices (the values of the vertices it
    // points at; the device keeps per-triangle records, so shared vertices need no
    // lookup), and consecutive triangles usually share a material
    const auto& geoms = scene.GetGeometries();
    const size_t G = geoms.size();
    pos.resize(9 * G);
    nrm.resize(9 * G);
    uv.resize(9 * G);
    idx.resize(3 * G);
    triMat.resize(G);
    shading.resize(G);
    const MaterialBase* lastMat = nullptr;
    int32_t lastIdx = -1;
    for (size_t i = 0; i < G; i++) {
        const auto* t = dynamic_cast<const Triangle*>(geoms[i]);
        if (!t) return fail(PT_ERR_UNSUPPORTED, "only triangle geometry is supported");
        const MaterialBase* m = t->GetMaterialPointer();
        if (!m) return fail(PT_ERR_INVALID_ARG, "geometry without material");
        int c = 0;
        for (const Vertex* v : t->GetVertices()) {
            const size_t k = 3 * i + c++;
            const float p3[9] = {v->pos.x, v->pos.y, v->pos.z, v->normal.x, v->normal.y, v->normal.z,
                                 v->uv.x, v->uv.y, v->uv.z};
            std::memcpy(&pos[3 * k], p3, 12);
            std::memcpy(&nrm[3 * k], p3 + 3, 12);
            std::memcpy(&uv[3 * k], p3 + 6, 12);
            idx[k] = (int32_t)k;
        }
        if (m != lastMat) {
            lastMat = m;
            lastIdx = addMaterial(m);
        }
        triMat[i] = lastIdx;
        shading[i] = t->GetShadingType() == ShadingTypes::Smooth ? 1 : 0;
    }
    if (!scene.GetLights().empty()) {
        std::unordered_map<const GeometryBase*, int32_t> lightSlot;
        for (size_t j = 0; j < scene.GetLights().size(); j++) lightSlot[scene.GetLights()[j]] = -1;
        for (size_t i = 0; i < G; i++) {
            auto it = lightSlot.find(geoms[i]);
            if (it != lightSlot.end()) it->second = (int32_t)i;  // the last occurrence, as before
        }
        for (const GeometryBase* l : scene.GetLights()) {
            const int32_t t = lightSlot[l];
            if (t < 0) return fail(PT_ERR_INVALID_ARG, "light is not a scene geometry");
            lights.push_back(t);
        }
    }
    if (mats.empty()) mats.push_back(pt_material{});  // an empty scene still needs one
    if (!texError.empty()) return fail(PT_ERR_INVALID_ARG, texError);

    pt_scene_desc d{};
    d.num_vertices = (uint32_t)(pos.size() / 3);
    d.positions = pos.data();
    d.normals = nrm.data();
    d.uvs = uv.data();
    d.num_triangles = (uint32_t)triMat.size();
    d.indices = idx.data();
    d.tri_material = triMat.data();
    d.tri_shading = shading.data();
    d.num_materials = (uint32_t)mats.size();
    d.materials = mats.data();
    d.num_lights = (uint32_t)lights.size();
    d.lights = lights.data();
    const Environment& env = scene.GetEnvironment();
    d.env_base_color[0] = env.GetBaseColor().x;
    d.env_base_color[1] = env.GetBaseColor().y;
    d.env_base_color[2] = env.GetBaseColor().z;
    d.env_z_rotation = env.GetZAxisRotation();
    if (env.GetTexture() && env.GetTexture()->IsValid()) {
        d.env_width = env.GetTexture()->GetWidth();
        d.env_height = env.GetTexture()->GetHeight();
        d.env_rgb = env.GetTexture()->GetRawDataPtr();
    }
    d.num_textures = (uint32_t)textures.size();
    d.textures = textures.data();
    pt_scene_id sid = 0;
    int rc = pt_scene_upload(m_ctx, &d, &sid);
    if (rc != PT_OK) return fail(rc, pt_last_error(m_ctx));

    pt_camera pc{};
    const Math::Vector3f* src[4] = {&cam->Position(), nullptr, nullptr, nullptr};
    const Math::Vector3f right = cam->Right(), up = cam->Up(), fwd = cam->Forward();
    src[1] = &right;
    src[2] = &up;
    src[3] = &fwd;
    float* dst[4] = {pc.pos, pc.right, pc.up, pc.forward};
    for (int k = 0; k < 4; k++) {
        dst[k][0] = src[k]->x;
        dst[k][1] = src[k]->y;
        dst[k][2] = src[k]->z;
    }
    pc.h_perf = cam->GetHPerf();
    pc.focus_dist = cam->GetFocusDist();
    pc.aperture = cam->GetApeture();

    const RenderSetting& rs = scene.GetRenderSetting();
    pt_settings st{};
    st.spp = rs.numSamplesPerPixel;
    st.max_bounces = rs.numMaxBounces;
    st.tile_width = rs.tileWidth;
    st.tile_height = rs.tileHeight;
    st.integrator = m_integrator;
    st.mode = m_mode;
    st.seed = m_seed;
    st.env_sampling = m_envSampling;
    st.denoising_spp = rs.numSppForDenoising;
    // the Rendered pass, then UV, DenoisingAlbedo and DenoisingNormal
    // (Petrichor.cpp:50-261), each at its own target's size
    const int32_t passes[Scene::AOVType::NumAOVTypes] = {-1, PT_AOV_UV, PT_AOV_DENOISING_ALBEDO,
                                                          PT_AOV_DENOISING_NORMAL};
    for (int a = Scene::AOVType::Rendered; a < Scene::AOVType::NumAOVTypes; a++) {
        Texture2D* tex = scene.GetTargetTexture((Scene::AOVType::Value)a);
        if (!tex) {
            if (a == Scene::AOVType::Rendered) std::cerr << "[Error] Target texture has not been set.\n";
            continue;
        }
        st.width = tex->GetWidth();
        st.height = tex->GetHeight();
        rc = a == Scene::AOVType::Rendered
               ? pt_render(m_ctx, sid, &pc, &st, tex->GetRawDataPtr())
               : pt_render_aov(m_ctx, sid, &pc, &st, passes[a], tex->GetRawDataPtr());
        if (rc != PT_OK) {
            fail(rc, pt_last_error(m_ctx));
            break;
        }
    }
    pt_scene_release(m_ctx, sid);
    if (m_callback) {
        RenderingResult r;
        r.totalSec = std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
        m_callback(r);
    }
}

}  // namespace Core
}  // namespace Petrichor
