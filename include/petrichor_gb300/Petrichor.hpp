// C++ scene/renderer API of the GB300 core, with the class and method names of
// the Petrichor renderer's own API (LibPetrichor/Core/Scene.h, Camera.h,
// Texture2D.h, Environment.h, Geometry/Vertex.h, Geometry/Triangle.h,
// Material/*.h, RenderSetting.h, Petrichor.h). Code written against that API
// switches by include path: scenes are built with the same calls and
// Petrichor::Render(scene) fills the Rendered target texture, through the C ABI
// in petrichor_gb300.h.
//
// Loaders: Scene::LoadAssets reads the reference's JSON scene format (materials,
// camera, env, assets; SceneLoader.cpp:17-297), Scene::LoadModel reads OBJ meshes
// (the reference uses Assimp; this is an own subset reader: v/vn/vt/f, one vertex per
// face corner, the first three corners of a polygon), Texture2D::Load reads PNG
// (colour textures linearised with a 2.2 power, as the reference does) and Radiance
// .hdr, and Texture2D::Save writes tone-mapped .png and .hdr (Texture2D.cpp:107-252).
// Material texture maps (Lambert albedo; GGX reflectance, roughness and normal maps)
// are rendered by every pass, and LoadAssets attaches the "color_tex" and
// "roughness_tex" maps of the JSON format.
//
// Differences, all additive: Petrichor::SetMode/SetIntegrator/SetSeed/SetEnvSampling
// choose the GB300 path (default: replay mode, SimplePathTracing, the reference's
// environment tables, i.e. the reference's own Render output bit for bit);
// Scene::SetRenderSetting sets settings without a
// file; Environment::SetTexture takes a texture from memory. The Rendered pass and
// the UV / DenoisingAlbedo / DenoisingNormal AOV passes are produced for the
// targets that are set, each equal to the reference's; only triangle geometry is
// accepted.
#pragma once

#include <array>
#include <cstdint>
#include <filesystem>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>

struct pt_context;

namespace Petrichor {
namespace Math {

struct Vector3f {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    constexpr Vector3f() = default;
    constexpr Vector3f(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
    static constexpr Vector3f Zero() { return {0.0f, 0.0f, 0.0f}; }
    static constexpr Vector3f One() { return {1.0f, 1.0f, 1.0f}; }
    static constexpr Vector3f UnitX() { return {1.0f, 0.0f, 0.0f}; }
    static constexpr Vector3f UnitY() { return {0.0f, 1.0f, 0.0f}; }
    static constexpr Vector3f UnitZ() { return {0.0f, 0.0f, 1.0f}; }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    Vector3f operator+(const Vector3f& v) const { return {x + v.x, y + v.y, z + v.z}; }
    Vector3f operator-(const Vector3f& v) const { return {x - v.x, y - v.y, z - v.z}; }
    Vector3f operator-() const { return {-x, -y, -z}; }
    Vector3f operator*(float c) const { return {x * c, y * c, z * c}; }
    Vector3f operator*(const Vector3f& v) const { return {x * v.x, y * v.y, z * v.z}; }
    Vector3f operator/(float c) const { return {x / c, y / c, z / c}; }
    float Length() const;
    Vector3f Normalized() const;
};
inline Vector3f operator*(float c, const Vector3f& v) { return v * c; }
inline float Dot(const Vector3f& a, const Vector3f& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vector3f Cross(const Vector3f& a, const Vector3f& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Math/AliasMethod.h:26-105: Walker's alias table over a discrete distribution, built
// here with Vose's linear construction (M. D. Vose, IEEE TSE 17(9), 1991). Sample(r0,
// r1) with r0, r1 uniform in [0, 1): column int(r0 n), then its own index when r1 is
// below the column's threshold, else its alias. The wavefront path's optional
// environment importance sampling (pt_settings.env_sampling) uses the same table.
class AliasMethod {
public:
    template <class T>
    void Construct(const std::vector<T>& distribution) {
        std::vector<double> w(distribution.size());
        for (size_t i = 0; i < w.size(); i++) w[i] = static_cast<double>(distribution[i]);
        Build(w);
    }
    int Sample(float r0, float r1) const {
        const int n = static_cast<int>(m_threshold.size());
        int i = static_cast<int>(r0 * static_cast<float>(n));
        i = i < 0 ? 0 : (i >= n ? n - 1 : i);
        return r1 < m_threshold[i] ? i : m_alias[i];
    }
    // the table: per column the probability of keeping it, and its alias
    const std::vector<float>& GetThresholds() const { return m_threshold; }
    const std::vector<int32_t>& GetAliases() const { return m_alias; }
    bool IsValid() const { return !m_threshold.empty(); }

private:
    void Build(const std::vector<double>& w) {
        m_threshold.assign(w.size(), 1.0f);
        m_alias.resize(w.size());
        double total = 0.0;
        for (double x : w) total += x > 0.0 ? x : 0.0;
        if (w.empty() || !(total > 0.0)) {
            m_threshold.clear();
            m_alias.clear();
            return;
        }
        const double n = static_cast<double>(w.size());
        std::vector<double> p(w.size());
        std::vector<int32_t> small, large;
        for (size_t i = 0; i < w.size(); i++) {
            m_alias[i] = static_cast<int32_t>(i);
            p[i] = (w[i] > 0.0 ? w[i] : 0.0) * n / total;
            (p[i] < 1.0 ? small : large).push_back(static_cast<int32_t>(i));
        }
        while (!small.empty() && !large.empty()) {
            const int32_t s = small.back(), l = large.back();
            small.pop_back();
            m_threshold[s] = static_cast<float>(p[s]);
            m_alias[s] = l;
            p[l] = (p[l] + p[s]) - 1.0;
            if (p[l] < 1.0) {
                large.pop_back();
                small.push_back(l);
            }
        }
        // what is left (large columns, and small ones from rounding) keeps itself
    }
    std::vector<float> m_threshold;
    std::vector<int32_t> m_alias;
};

}  // namespace Math

using Color3f = Math::Vector3f;

struct RenderingResult {
    float totalSec;
};

namespace Core {

enum class MaterialTypes { Lambert, Glass, Emission, Glossy, Mix };
enum class ShadingTypes { Flat, Smooth };

struct RenderSetting {
    int outputWidth = 1280;
    int outputHeight = 720;
    int numSamplesPerPixel = 128;
    int numSppForDenoising = 128;
    int numMaxBounces = 16;
    int tileWidth = 16;
    int tileHeight = 16;
    int numThreads = 0;
};

class MaterialBase {
public:
    virtual ~MaterialBase() = default;
    virtual MaterialTypes GetMaterialType() const = 0;
    // MaterialBase.h:52-62; Lambert reads it (off: uniform hemisphere sampling,
    // Lambert.cpp:40-47,85-107), the other materials ignore it
    void EnableImportanceSampling(bool isEnabled) { m_isImportanceSamplingEnabled = isEnabled; }
    bool IsImportanceSamplingEnabled() const { return m_isImportanceSamplingEnabled; }

private:
    bool m_isImportanceSamplingEnabled = true;
};

class Texture2D;

// Texture maps are sampled bilinearly with wrap-around at the shading point's uv;
// the texture must outlive the render (the scene keeps pointers, as the reference does).
class Lambert : public MaterialBase {
public:
    explicit Lambert(const Color3f& kd) : m_kd(kd) {}
    MaterialTypes GetMaterialType() const override { return MaterialTypes::Lambert; }
    const Color3f& GetKd() const { return m_kd; }
    // Lambert.h:37-41: albedo = kd * texel
    void SetTexAlbedo(const Texture2D* texAlbedo) { m_texAlbedo = texAlbedo; }
    const Texture2D* GetTexAlbedo() const { return m_texAlbedo; }

private:
    Color3f m_kd;
    const Texture2D* m_texAlbedo = nullptr;
};

class GGX : public MaterialBase {
public:
    GGX(const Color3f& f0, float roughness = 1.0f) : m_f0(f0), m_roughness(roughness) {}
    MaterialTypes GetMaterialType() const override { return MaterialTypes::Glossy; }
    const Color3f& GetReflectance() const { return m_f0; }
    float GetRoughness() const { return m_roughness; }
    // GGX.h:43-93: reflectance = f0 * texel; alpha = (strength * luminance(texel))^2;
    // tangent-space normal map blended by its strength (clamped to [0, 1])
    void SetF0Texture(const Texture2D* texture) { m_f0Map = texture; }
    void SetRoughnessMap(const Texture2D* roughnessMap) { m_roughnessMap = roughnessMap; }
    void SetNormalMap(const Texture2D* normalMap) { m_normalMap = normalMap; }
    void SetRoughnessMapStrength(float strength) { m_roughnessMapStrength = strength; }
    void SetNormalMapStrength(float strength) {
        m_normalMapStrength = strength < 0.0f ? 0.0f : (strength > 1.0f ? 1.0f : strength);
    }
    const Texture2D* GetF0Texture() const { return m_f0Map; }
    const Texture2D* GetRoughnessMap() const { return m_roughnessMap; }
    const Texture2D* GetNormalMap() const { return m_normalMap; }
    float GetRoughnessMapStrength() const { return m_roughnessMapStrength; }
    float GetNormalMapStrength() const { return m_normalMapStrength; }

private:
    Color3f m_f0;
    float m_roughness;
    const Texture2D* m_f0Map = nullptr;
    const Texture2D* m_roughnessMap = nullptr;
    const Texture2D* m_normalMap = nullptr;
    float m_roughnessMapStrength = 1.0f;
    float m_normalMapStrength = 1.0f;
};

class Glass : public MaterialBase {
public:
    struct IOR {
        static constexpr float Water = 1.333f;
    };
    Glass() = default;
    explicit Glass(const Color3f& color, float ior) noexcept : m_color(color), m_ior(ior) {}
    MaterialTypes GetMaterialType() const override { return MaterialTypes::Glass; }
    float GetIOR() const { return m_ior; }
    const Color3f& GetColor() const { return m_color; }

private:
    Color3f m_color = Color3f::One();
    float m_ior = IOR::Water;
};

class Emission : public MaterialBase {
public:
    Emission(const Color3f& color) : m_color(color) {}
    MaterialTypes GetMaterialType() const override { return MaterialTypes::Emission; }
    const Color3f& GetLightColor() const { return m_color; }

private:
    Color3f m_color;
};

class MixMaterial : public MaterialBase {
public:
    MixMaterial(const MaterialBase* mat0, const MaterialBase* mat1, float mix)
        : m_mat0(mat0), m_mat1(mat1), m_mix(mix) {}
    MaterialTypes GetMaterialType() const override { return MaterialTypes::Mix; }
    const MaterialBase* GetMat0() const { return m_mat0; }
    const MaterialBase* GetMat1() const { return m_mat1; }
    float GetMix() const { return m_mix; }

private:
    const MaterialBase* m_mat0;
    const MaterialBase* m_mat1;
    float m_mix;
};

struct Vertex {
    constexpr Vertex() = default;
    Vertex(float x, float y, float z) : pos{x, y, z} {}
    Vertex(const Math::Vector3f& p, const Math::Vector3f& n, const Math::Vector3f& t)
        : pos(p), normal(n), uv(t) {}
    Math::Vector3f pos;
    Math::Vector3f normal = Math::Vector3f::UnitZ();
    Math::Vector3f uv;
};

class GeometryBase {
public:
    virtual ~GeometryBase() = default;
    void SetMaterial(const MaterialBase* material) { m_material = material; }
    const MaterialBase* GetMaterialPointer() const { return m_material; }

protected:
    const MaterialBase* m_material = nullptr;
};

class Triangle : public GeometryBase {
public:
    explicit Triangle(ShadingTypes shadingType) : m_shadingType(shadingType) {}
    Triangle(const Vertex* v0, const Vertex* v1, const Vertex* v2) { SetVertices(v0, v1, v2); }
    Triangle(const Vertex* v0, const Vertex* v1, const Vertex* v2, ShadingTypes shadingType)
        : Triangle(v0, v1, v2) {
        m_shadingType = shadingType;
    }
    void SetVertices(const Vertex* v0, const Vertex* v1, const Vertex* v2) { m_vertices = {v0, v1, v2}; }
    const std::array<const Vertex*, 3>& GetVertices() const { return m_vertices; }
    ShadingTypes GetShadingType() const { return m_shadingType; }

private:
    std::array<const Vertex*, 3> m_vertices{};
    ShadingTypes m_shadingType = ShadingTypes::Flat;
};

class Texture2D {
public:
    enum class TextureColorType { Color, NonColor };
    Texture2D() : Texture2D(0, 0) {}
    Texture2D(int width, int height);
    // ".hdr": Radiance RGBE (flat or run-length encoded scanlines), or the raw container
    // "PTRAWF32", uint32 width, uint32 height, RGB float32 rows.
    bool Load(const std::filesystem::path& path, TextureColorType type = TextureColorType::Color);
    // ".png": ACES + the reference's tone curve, 8-bit RGB; ".hdr": Radiance RGBE.
    void Save(const std::filesystem::path& path) const;
    void Clear(const Color3f& color = Color3f::Zero());
    Color3f GetPixel(int i, int j) const;
    // Texture2D.h:27-71: point or bilinear lookup at texel coordinates (x = u * width, no
    // half-texel shift, edges clamped), and at wrapped uv
    enum class InterplationTypes { Point, Bilinear };
    Color3f GetPixel(float x, float y, InterplationTypes type = InterplationTypes::Bilinear) const;
    Color3f GetPixelByUV(float u, float v, InterplationTypes type = InterplationTypes::Bilinear) const;
    void SetPixel(int i, int j, const Color3f& color);
    int GetWidth() const { return m_width; }
    int GetHeight() const { return m_height; }
    bool IsValid() const { return m_isLoaded && m_width > 0 && m_height > 0; }
    const float* GetRawDataPtr() const { return m_pixels.data(); }
    float* GetRawDataPtr() { return m_pixels.data(); }
    // Marks the contents as image data (what Load does for a file).
    void SetLoaded(bool loaded) { m_isLoaded = loaded; }

private:
    int m_width = 0, m_height = 0;
    std::vector<float> m_pixels;
    bool m_isLoaded = false;
};

class Mesh {
public:
    // OBJ subset (see the header comment); every triangle gets `material` and `shadingType`.
    void Load(const std::filesystem::path& path, const MaterialBase* material,
              ShadingTypes shadingType = ShadingTypes::Flat);
    const std::vector<Triangle>& GetTriangles() const { return m_triangles; }

private:
    std::vector<Vertex> m_vertices;
    std::vector<Triangle> m_triangles;
};

class Environment {
public:
    void Load(const std::filesystem::path& path);
    void SetTexture(const Texture2D& texture);
    void SetBaseColor(const Color3f& baseColor) { m_baseColor = baseColor; }
    void SetZAxisRotation(float angle) { m_ZAxisRotation = angle; }
    const Color3f& GetBaseColor() const { return m_baseColor; }
    float GetZAxisRotation() const { return m_ZAxisRotation; }
    const Texture2D* GetTexture() const { return m_tex.get(); }

private:
    std::shared_ptr<Texture2D> m_tex;
    Color3f m_baseColor;
    float m_ZAxisRotation = 0.0f;
};

class Camera {
public:
    Camera() = default;
    Camera(const Math::Vector3f& pos, const Math::Vector3f& dir);
    void SetPosition(const Math::Vector3f& pos) { m_pos = pos; }
    void SetFocalLength(float focalLength);
    void FocusTo(const Math::Vector3f& target);
    void SetFOV(float fov);
    void SetViewDir(const Math::Vector3f& dir);
    void LookAt(const Math::Vector3f& target);
    float GetFocalLength() const { return m_sensorHeight / m_hPerf; }
    float GetApeture() const { return m_apeture; }
    void SetApeture(float apeture) { m_apeture = apeture; }
    void SetFNumber(float fNumber) { m_apeture = GetFocalLength() / fNumber; }
    float GetFOV() const;
    float GetLensArea() const;
    Math::Vector3f Right() const { return m_right; }
    Math::Vector3f Up() const { return m_up; }
    Math::Vector3f Forward() const { return m_forward; }
    const Math::Vector3f& Position() const { return m_pos; }
    float GetHPerf() const { return m_hPerf; }
    float GetFocusDist() const { return m_focusDist; }

private:
    Math::Vector3f m_pos, m_right, m_up, m_forward;
    float m_focusDist = 1.0f;
    float m_sensorHeight = 24e-3f;
    float m_hPerf = 24e-3f / 55e-3f;
    float m_apeture = 25e-3f;
};

struct TextureHandle {  // Scene.h:24-27
    std::string filePath;
};

class Scene {
public:
    struct AOVType {
        enum Value { Rendered, UV, DenoisingAlbedo, DenoisingNormal, NumAOVTypes };
    };

    void AppendGeometry(const GeometryBase* geometry) { m_geometries.push_back(geometry); }
    void AppendLight(const GeometryBase* geometry) { m_lights.push_back(geometry); }
    void AppendMesh(const Mesh& mesh) {
        for (const Triangle& t : mesh.GetTriangles()) AppendGeometry(&t);
    }
    void AppendLightMesh(const Mesh& mesh) {
        for (const Triangle& t : mesh.GetTriangles()) {
            AppendGeometry(&t);
            AppendLight(&t);
        }
    }
    // Loads an OBJ with the "default" material (or the named one), smooth shading
    // (Scene.cpp:29-52). The scene keeps the mesh.
    void LoadModel(const std::filesystem::path& path);
    void LoadModel(const std::filesystem::path& path, std::string_view materialName);
    // The reference's JSON scene file (SceneLoaderJson, SceneLoader.cpp:17-297).
    void LoadAssets(const std::filesystem::path& path);
    const std::vector<const GeometryBase*>& GetGeometries() const { return m_geometries; }
    const std::vector<const GeometryBase*>& GetLights() const { return m_lights; }
    const Camera* GetMainCamera() const { return m_mainCamera.get(); }
    void SetMainCamera(std::unique_ptr<Camera> camera) { m_mainCamera = std::move(camera); }
    void RegisterMaterial(std::string_view name, std::unique_ptr<const MaterialBase> material) {
        m_materials[std::string(name)] = std::move(material);
    }
    const MaterialBase* GetMaterial(std::string_view name) { return m_materials[std::string(name)].get(); }
    // Scene.h:131-158: textures kept by the scene under their file path; the first
    // registration of a path wins, and the pointers stay valid for the scene's life.
    TextureHandle RegisterTexture(const std::filesystem::path& filePath, const Texture2D& texture) {
        m_textures.emplace(filePath.string(), texture);
        return TextureHandle{filePath.string()};
    }
    const Texture2D* GetTexture(const TextureHandle& handle) {
        auto it = m_textures.find(handle.filePath);
        return it == m_textures.end() ? nullptr : &it->second;
    }
    const Environment& GetEnvironment() const { return m_environment; }
    void SetEnvironment(const Environment& environment) { m_environment = environment; }
    void SetTargetTexture(AOVType::Value type, Texture2D* target) { m_targets[type] = target; }
    Texture2D* GetTargetTexture(AOVType::Value type) const { return m_targets[type]; }
    // JSON keys of RenderSettingLoaderJson; a ".toml" file uses the settings.* keys.
    void LoadRenderSetting(const std::filesystem::path& path);
    void SetRenderSetting(const RenderSetting& setting) { m_renderSetting = setting; }
    const RenderSetting& GetRenderSetting() const { return m_renderSetting; }

private:
    std::vector<const GeometryBase*> m_geometries, m_lights;
    std::unordered_map<std::string, std::unique_ptr<const MaterialBase>> m_materials;
    std::map<std::string, Texture2D> m_textures;
    Environment m_environment;
    std::unique_ptr<Camera> m_mainCamera;
    std::array<Texture2D*, AOVType::NumAOVTypes> m_targets{};
    RenderSetting m_renderSetting;
    std::vector<std::unique_ptr<Mesh>> m_meshes;
};

class Petrichor {
public:
    Petrichor();
    ~Petrichor();
    void Render(const Scene& scene);
    void SetRenderCallback(const std::function<void(const RenderingResult&)>& cb) { m_callback = cb; }
    uint32_t GetNumRenderedTiles() const;
    uint32_t GetNumTiles() const;
    // GB300 path selection: mode PT_MODE_REPLAY / PT_MODE_WAVEFRONT, integrator
    // PT_INTEGRATOR_SIMPLE (the reference's Render) / PT_INTEGRATOR_PT, stream seed.
    void SetMode(int mode) { m_mode = mode; }
    void SetIntegrator(int integrator) { m_integrator = integrator; }
    void SetSeed(uint32_t seed) { m_seed = seed; }
    // Environment next-event sampling: PT_ENV_SAMPLING_REFERENCE, or PT_ENV_SAMPLING_ALIAS
    // (wavefront mode; an alias table over the map, a different unbiased estimator).
    void SetEnvSampling(int sampling) { m_envSampling = sampling; }
    // Status of the last Render (PT_OK or a PT_ERR_* code) and its message.
    int GetLastStatus() const { return m_lastStatus; }
    const std::string& GetLastError() const { return m_lastError; }

private:
    pt_context* m_ctx = nullptr;
    std::function<void(const RenderingResult&)> m_callback;
    int m_mode = 0, m_integrator = 0, m_envSampling = 0;
    uint32_t m_seed = 1;
    int m_lastStatus = 0;
    std::string m_lastError;
};

// Core/Denoiser/IntelOpenImageDenoiser.h:10-38, with the same calls. Intel Open Image
// Denoise is not part of this library: Denoise runs the GPU filter of pt_denoise
// (edge-avoiding à-trous, guided by the albedo and normal AOVs when given), so the
// images differ from the reference's. On an error the message goes to stderr and the
// returned texture is black, as the reference leaves its output on an OIDN error.
class IntelOpenImageDenoiser {
public:
    struct ImageType {
        enum Type { Color, Albedo, Normal };
    };
    IntelOpenImageDenoiser();
    ~IntelOpenImageDenoiser();
    IntelOpenImageDenoiser(const IntelOpenImageDenoiser&) = delete;
    IntelOpenImageDenoiser& operator=(const IntelOpenImageDenoiser&) = delete;
    Texture2D Denoise(const Texture2D& color, bool isHDR);
    Texture2D Denoise(const Texture2D& color, const Texture2D& albedo, const Texture2D& normal,
                      bool isHDR);

private:
    Texture2D Run(const Texture2D& color, const Texture2D* albedo, const Texture2D* normal, bool isHDR);
    pt_context* m_ctx = nullptr;
};

}  // namespace Core
}  // namespace Petrichor
