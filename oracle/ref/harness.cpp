// Oracle harness around the reference renderer (test infrastructure only).
//
// Builds a scene from a .ptscene file through the reference's public C++ API
// (Scene::AppendGeometry/AppendLight/RegisterMaterial/SetMainCamera/
// SetEnvironment/SetTargetTexture/LoadRenderSetting, Core/Scene.h:60-218) and
// runs the reference code unchanged:
//   film  : Petrichor::Render (SimplePathTracing, Core/Petrichor.cpp:35-102), or
//           for the MIS integrator the same tile loop with PathTracing
//           (Core/Integrator/PathTracing.cpp:20-200), seeds as Petrichor.cpp:72-77
//   hits  : Camera::GenerateRay + BinnedSAHBVH::Intersect for one ray per pixel,
//           with the triangle index, distance and number of triangle tests
//   bvh   : BinnedSAHBVH::Build, dumping its nodes and primitive order
//   env   : Environment::ImportanceSampling / GetImportanceSamplingPDF / GetColor
// Output is raw little-endian binary read by tests/golden/make_golden.py.
#include "Core/Accel/BinnedSAHBVH.h"
#include "Core/Camera.h"
#include "Core/Environment.h"
#include "Core/Geometry/Triangle.h"
#include "Core/Geometry/Vertex.h"
#include "Core/Integrator/PathTracing.h"
#include "Core/Material/Emission.h"
#include "Core/Material/GGX.h"
#include "Core/Material/Glass.h"
#include "Core/Material/Lambert.h"
#include "Core/Material/MixMaterial.h"
#include "Core/Petrichor.h"
#include "Core/Sampler/RandomSampler1D.h"
#include "Core/Sampler/RandomSampler2D.h"
#include "Core/Scene.h"
#include "Core/Texture2D.h"
#include "Core/Thread/ThreadPool.h"
#include "Core/TileManager.h"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

using namespace Petrichor;
using namespace Petrichor::Core;

// ---- read access to BinnedSAHBVH's private node arrays (explicit-instantiation idiom)
struct NodesTag {};
struct PrimIDsTag {};
struct DepthTag {};
template <typename Tag, auto M>
struct Steal {
    friend auto Get(Tag) { return M; }
};
auto Get(NodesTag);
auto Get(PrimIDsTag);
auto Get(DepthTag);
template struct Steal<NodesTag, &BinnedSAHBVH::m_nodes>;
template struct Steal<PrimIDsTag, &BinnedSAHBVH::m_primitiveIDs>;
template struct Steal<DepthTag, &BinnedSAHBVH::m_maxBVHDepth>;

// ---- a Triangle that counts its ray tests (Intersect is virtual, GeometryBase.h:31-32)
thread_local long g_numTriangleTests = 0;
class CountingTriangle : public Triangle {
public:
    using Triangle::Triangle;
    std::optional<HitInfo> Intersect(const Ray& ray) const override {
        g_numTriangleTests++;
        return Triangle::Intersect(ray);
    }
};

struct Reader {
    std::vector<char> buf;
    size_t off = 0;
    explicit Reader(const std::string& path) {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw std::runtime_error("cannot open " + path);
        buf.assign(std::istreambuf_iterator<char>(f), {});
    }
    template <typename T>
    T get() {
        T v;
        take(&v, sizeof(T));
        return v;
    }
    void take(void* dst, size_t n) {
        if (off + n > buf.size()) throw std::runtime_error("truncated scene");
        std::memcpy(dst, buf.data() + off, n);
        off += n;
    }
};

struct Loaded {
    int settings[8];
    std::vector<Vertex> vertices;
    std::vector<CountingTriangle> triangles;
    std::unique_ptr<Scene> scene = std::make_unique<Scene>();
    std::unique_ptr<Texture2D> film;
    std::vector<const MaterialBase*> materials;
    int integrator = 0;
    int denoisingSpp = 1;
    std::vector<std::unique_ptr<Texture2D>> textures;  // material texture maps
};

static Math::Vector3f V3(const float* p) { return Math::Vector3f(p[0], p[1], p[2]); }

static void Load(const std::string& path, const std::string& tmpPrefix, Loaded& L) {
    Reader r(path);
    char magic[8];
    r.take(magic, 8);
    if (std::memcmp(magic, "PTSCENE1", 8) != 0) throw std::runtime_error("bad magic");
    for (int i = 0; i < 8; i++) L.settings[i] = r.get<int32_t>();
    L.integrator = L.settings[7];
    {
        const std::string sp = tmpPrefix + ".settings.json";
        std::ofstream s(sp);
        s << "{\"outputWidth\": " << L.settings[0] << ", \"outputHeight\": " << L.settings[1]
          << ", \"spp\": " << L.settings[2] << ", \"denoising_spp\": " << L.denoisingSpp
          << ", \"maxBounces\": "
          << L.settings[3] << ", \"tileWidth\": " << L.settings[4]
          << ", \"tileHeight\": " << L.settings[5] << ", \"numThreads\": " << L.settings[6]
          << "}\n";
        s.close();
        L.scene->LoadRenderSetting(sp);
    }
    float cam[12];
    r.take(cam, sizeof(cam));
    const uint32_t hasFocus = r.get<uint32_t>();
    {
        auto c = std::make_unique<Camera>(V3(cam + 0), V3(cam + 3));
        if (cam[6] > 0.0f) c->SetFOV(cam[6]);
        else c->SetFocalLength(cam[7]);
        if (hasFocus) c->FocusTo(V3(cam + 8));
        c->SetApeture(cam[11]);
        L.scene->SetMainCamera(std::move(c));
    }
    float envf[4];
    r.take(envf, sizeof(envf));
    const int32_t ew = r.get<int32_t>(), eh = r.get<int32_t>();
    (void)r.get<uint32_t>();  // importance-sampling flag: always on in the reference
    Environment env;
    env.SetBaseColor(V3(envf));
    env.SetZAxisRotation(envf[3]);
    if (ew > 0 && eh > 0) {
        std::vector<float> px((size_t)ew * eh * 3);
        r.take(px.data(), px.size() * 4);
        const std::string hp = tmpPrefix + ".env.hdr";
        std::ofstream h(hp, std::ios::binary);
        const uint32_t dims[2] = {(uint32_t)ew, (uint32_t)eh};
        h.write("PTRAWF32", 8);
        h.write((const char*)dims, 8);
        h.write((const char*)px.data(), px.size() * 4);
        h.close();
        env.Load(hp);
    }
    L.scene->SetEnvironment(env);

    const uint32_t M = r.get<uint32_t>();
    std::vector<float> mf((size_t)M * 8);
    std::vector<int32_t> mi((size_t)M * 4);
    r.take(mf.data(), mf.size() * 4);
    r.take(mi.data(), mi.size() * 4);
    L.materials.assign(M, nullptr);
    std::vector<Lambert*> lamberts(M, nullptr);
    std::vector<GGX*> ggxs(M, nullptr);
    for (int pass = 0; pass < 2; pass++) {
        for (uint32_t k = 0; k < M; k++) {
            const float* f = &mf[k * 8];
            const int32_t* q = &mi[k * 4];
            std::unique_ptr<const MaterialBase> m;
            if (pass == 0) {
                switch (q[0]) {
                case 0: {
                    auto l = std::make_unique<Lambert>(V3(f));
                    lamberts[k] = l.get();
                    m = std::move(l);
                    break;
                }
                case 1: m = std::make_unique<Glass>(V3(f), f[4]); break;
                case 2: m = std::make_unique<Emission>(V3(f)); break;
                case 3: {
                    auto g = std::make_unique<GGX>(V3(f), f[3]);
                    ggxs[k] = g.get();
                    m = std::move(g);
                    break;
                }
                default: break;
                }
            } else if (q[0] == 4) {
                m = std::make_unique<MixMaterial>(L.materials.at(q[1]), L.materials.at(q[2]), f[5]);
            }
            if (m) {
                const std::string name = "m" + std::to_string(k);
                L.materials[k] = m.get();
                L.scene->RegisterMaterial(name, std::move(m));
            }
        }
    }

    const uint32_t V = r.get<uint32_t>();
    std::vector<float> pos((size_t)V * 3), nrm((size_t)V * 3), uv((size_t)V * 3);
    r.take(pos.data(), pos.size() * 4);
    r.take(nrm.data(), nrm.size() * 4);
    r.take(uv.data(), uv.size() * 4);
    L.vertices.reserve(V);
    for (uint32_t i = 0; i < V; i++)
        L.vertices.emplace_back(V3(&pos[i * 3]), V3(&nrm[i * 3]), V3(&uv[i * 3]));
    const uint32_t T = r.get<uint32_t>();
    std::vector<int32_t> idx((size_t)T * 3), tm(T);
    std::vector<uint8_t> sh(T + ((4 - T % 4) % 4));
    r.take(idx.data(), idx.size() * 4);
    r.take(tm.data(), tm.size() * 4);
    r.take(sh.data(), sh.size());
    L.triangles.reserve(T);
    for (uint32_t t = 0; t < T; t++) {
        L.triangles.emplace_back(&L.vertices[idx[t * 3]], &L.vertices[idx[t * 3 + 1]],
                                 &L.vertices[idx[t * 3 + 2]],
                                 sh[t] ? ShadingTypes::Smooth : ShadingTypes::Flat);
        L.triangles.back().SetMaterial(L.materials.at(tm[t]));
    }
    for (uint32_t t = 0; t < T; t++) L.scene->AppendGeometry(&L.triangles[t]);
    const uint32_t NL = r.get<uint32_t>();
    for (uint32_t i = 0; i < NL; i++) L.scene->AppendLight(&L.triangles.at(r.get<int32_t>()));
    // optional texture maps: loaded through Texture2D::Load of raw .hdr files and attached
    // with the materials' setters (Lambert::SetTexAlbedo, GGX::SetF0Texture/SetRoughnessMap/
    // SetNormalMap and the map strengths)
    if (r.off < r.buf.size()) {
        const uint32_t NT = r.get<uint32_t>();
        for (uint32_t k = 0; k < NT; k++) {
            const int32_t tw = r.get<int32_t>(), th = r.get<int32_t>();
            std::vector<float> px((size_t)tw * th * 3);
            r.take(px.data(), px.size() * 4);
            const std::string tp = tmpPrefix + ".tex" + std::to_string(k) + ".hdr";
            std::ofstream h(tp, std::ios::binary);
            const uint32_t dims[2] = {(uint32_t)tw, (uint32_t)th};
            h.write("PTRAWF32", 8);
            h.write((const char*)dims, 8);
            h.write((const char*)px.data(), px.size() * 4);
            h.close();
            auto t = std::make_unique<Texture2D>();
            if (!t->Load(tp, Texture2D::TextureColorType::NonColor)) throw std::runtime_error("texture");
            std::remove(tp.c_str());
            L.textures.push_back(std::move(t));
        }
        auto tex = [&](uint32_t refs, int j) -> const Texture2D* {
            const int id = (int)((refs >> (8 * j)) & 255) - 1;
            return id >= 0 ? L.textures.at(id).get() : nullptr;
        };
        for (uint32_t k = 0; k < M; k++) {
            const uint32_t refs = (uint32_t)mi[k * 4 + 3];
            if (lamberts[k] && tex(refs, 0)) lamberts[k]->SetTexAlbedo(tex(refs, 0));
            if (ggxs[k]) {
                if (tex(refs, 1)) ggxs[k]->SetF0Texture(tex(refs, 1));
                if (tex(refs, 2)) {
                    ggxs[k]->SetRoughnessMap(tex(refs, 2));
                    ggxs[k]->SetRoughnessMapStrength(mf[k * 8 + 6]);
                }
                if (tex(refs, 3)) {
                    ggxs[k]->SetNormalMap(tex(refs, 3));
                    ggxs[k]->SetNormalMapStrength(mf[k * 8 + 7]);
                }
            }
        }
    }
    // optional per-material flags: bit 0 = MaterialBase::EnableImportanceSampling(false)
    if (r.off < r.buf.size()) {
        const uint32_t NM = r.get<uint32_t>();
        if (NM != M) throw std::runtime_error("material flag count");
        for (uint32_t k = 0; k < NM; k++) {
            const bool off = (r.get<uint32_t>() & 1u) != 0;
            if (lamberts[k]) lamberts[k]->EnableImportanceSampling(!off);
            if (ggxs[k]) ggxs[k]->EnableImportanceSampling(!off);
        }
    }

    L.film = std::make_unique<Texture2D>(L.settings[0], L.settings[1]);
    L.scene->SetTargetTexture(Scene::AOVType::Rendered, L.film.get());
}

static void WriteAll(const std::string& path, const void* p, size_t n) {
    std::ofstream f(path, std::ios::binary);
    f.write((const char*)p, (std::streamsize)n);
    if (!f) throw std::runtime_error("write failed: " + path);
}

static double Now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Rendered pass with PathTracing: the tile loop of Petrichor.cpp:62-95 with its seeds.
static void RenderPathTracing(const Scene& scene, const AccelBase& accel, Texture2D* target) {
    PathTracing pt;
    const TileManager tm(target->GetWidth(), target->GetHeight(),
                         scene.GetRenderSetting().tileWidth, scene.GetRenderSetting().tileHeight);
    ThreadPool pool(scene.GetRenderSetting().numThreads);
    int tileIndex = 0;
    for (const TileManager::Tile& tile : tm.GetTiles()) {
        pool.Push([&, tile, tileIndex](size_t) {
            RandomSampler1D s1(tileIndex);
            RandomSampler2D s2(tileIndex, tileIndex + 1);
            for (int y = tile.y; y < tile.y + tile.height; y++)
                for (int x = tile.x; x < tile.x + tile.width; x++)
                    pt.Render(x, y, scene, accel, target, s1, s2);
        });
    }
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr,
                     "usage: %s film|hits|bvh|env <scene.ptscene> <out.bin> [args]\n", argv[0]);
        return 2;
    }
    const std::string mode = argv[1], scenePath = argv[2], out = argv[3];
    try {
        Loaded L;
        if (mode == "aov" && argc > 4) L.denoisingSpp = std::stoi(argv[4]);
        Load(scenePath, out, L);
        const Scene& scene = *L.scene;
        if (mode == "film") {
            double t0 = Now();
            BinnedSAHBVH bvh;
            bvh.Build(scene);
            double t1 = Now();
            double t2, t3;
            if (L.integrator == 0) {
                Core::Petrichor renderer;
                t2 = Now();
                renderer.Render(scene);  // rebuilds the BVH itself (Petrichor.cpp:41-45)
                t3 = Now();
            } else {
                t2 = Now();
                RenderPathTracing(scene, bvh, L.film.get());
                t3 = Now();
            }
            const int W = L.film->GetWidth(), H = L.film->GetHeight();
            WriteAll(out, L.film->GetRawDataPtr(), (size_t)W * H * 3 * 4);
            unsigned nthreads = scene.GetRenderSetting().numThreads;
            if (nthreads == 0) nthreads = std::thread::hardware_concurrency();
            std::printf("{\"bvh_build_s\": %.6f, \"render_s\": %.6f, \"threads\": %u, "
                        "\"integrator\": %d}\n",
                        t1 - t0, t3 - t2, nthreads, L.integrator);
        } else if (mode == "hits") {
            const unsigned seedA = argc > 4 ? std::stoul(argv[4]) : 7u;
            const unsigned seedB = argc > 5 ? std::stoul(argv[5]) : 11u;
            BinnedSAHBVH bvh;
            bvh.Build(scene);
            const int W = L.settings[0], H = L.settings[1];
            RandomSampler2D s2(seedA, seedB);
            std::vector<float> rays((size_t)W * H * 8);
            std::vector<int32_t> hits((size_t)W * H * 2);
            const Camera* cam = scene.GetMainCamera();
            for (int y = 0; y < H; y++)
                for (int x = 0; x < W; x++) {
                    const size_t k = (size_t)y * W + x;
                    const Ray ray = cam->GenerateRay(x, y, W, H, s2);
                    g_numTriangleTests = 0;
                    const auto h = static_cast<const AccelBase&>(bvh).Intersect(ray, scene);
                    float* rr = &rays[k * 8];
                    rr[0] = ray.o.x; rr[1] = ray.o.y; rr[2] = ray.o.z;
                    rr[3] = ray.dir.x; rr[4] = ray.dir.y; rr[5] = ray.dir.z;
                    rr[6] = h ? h->distance : -1.0f;
                    rr[7] = ray.throughput.x;
                    hits[k * 2] = h ? (int32_t)(static_cast<const CountingTriangle*>(h->hitObj) -
                                                L.triangles.data())
                                    : -1;
                    hits[k * 2 + 1] = (int32_t)g_numTriangleTests;
                }
            std::vector<char> blob(rays.size() * 4 + hits.size() * 4);
            std::memcpy(blob.data(), rays.data(), rays.size() * 4);
            std::memcpy(blob.data() + rays.size() * 4, hits.data(), hits.size() * 4);
            WriteAll(out, blob.data(), blob.size());
        } else if (mode == "bvh") {
            BinnedSAHBVH bvh;
            const double t0 = Now();
            bvh.Build(scene);
            const double t1 = Now();
            const auto& nodes = bvh.*Get(NodesTag{});
            const auto& ids = bvh.*Get(PrimIDsTag{});
            std::vector<char> blob;
            auto put = [&](const void* p, size_t n) {
                blob.insert(blob.end(), (const char*)p, (const char*)p + n);
            };
            const int32_t nn = (int32_t)nodes.size(), ni = (int32_t)ids.size(),
                          depth = bvh.*Get(DepthTag{});
            put(&nn, 4);
            put(&ni, 4);
            put(&depth, 4);
            for (const auto& n : nodes) {
                const float b[6] = {n.boundary.lower.x, n.boundary.lower.y, n.boundary.lower.z,
                                    n.boundary.upper.x, n.boundary.upper.y, n.boundary.upper.z};
                const int32_t q[5] = {n.childIndicies[0], n.childIndicies[1], n.primIndexBegin,
                                      n.primIndexEnd, n.isLeaf ? 1 : 0};
                put(b, 24);
                put(q, 20);
            }
            put(ids.data(), ids.size() * 4);
            WriteAll(out, blob.data(), blob.size());
            std::printf("{\"bvh_build_s\": %.6f, \"nodes\": %d}\n", t1 - t0, nn);
        } else if (mode == "aov") {
            // the AOV passes of Petrichor::Render (Core/Petrichor.cpp:104-261), Rendered skipped
            const int W = L.settings[0], H = L.settings[1];
            Texture2D uv(W, H), albedo(W, H), normal(W, H);
            L.scene->SetTargetTexture(Scene::AOVType::Rendered, nullptr);
            L.scene->SetTargetTexture(Scene::AOVType::UV, &uv);
            L.scene->SetTargetTexture(Scene::AOVType::DenoisingAlbedo, &albedo);
            L.scene->SetTargetTexture(Scene::AOVType::DenoisingNormal, &normal);
            Core::Petrichor renderer;
            renderer.Render(scene);
            const size_t n = (size_t)W * H * 3;
            std::vector<float> o(3 * n);
            std::memcpy(o.data(), uv.GetRawDataPtr(), n * 4);
            std::memcpy(o.data() + n, albedo.GetRawDataPtr(), n * 4);
            std::memcpy(o.data() + 2 * n, normal.GetRawDataPtr(), n * 4);
            WriteAll(out, o.data(), o.size() * 4);
        } else if (mode == "env") {
            const int n = argc > 4 ? std::stoi(argv[4]) : 4096;
            RandomSampler2D s2(3, 4);
            const Environment& env = scene.GetEnvironment();
            std::vector<float> o((size_t)n * 8);
            for (int i = 0; i < n; i++) {
                float pdf = 0.0f;
                const Math::Vector3f d = env.ImportanceSampling(s2, &pdf);
                const Color3f c = env.GetColor(d);
                float* q = &o[(size_t)i * 8];
                q[0] = d.x; q[1] = d.y; q[2] = d.z; q[3] = pdf;
                q[4] = env.GetImportanceSamplingPDF(d);
                q[5] = c.x; q[6] = c.y; q[7] = c.z;
            }
            WriteAll(out, o.data(), o.size() * 4);
        } else {
            std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
            return 2;
        }
        std::remove((out + ".settings.json").c_str());
        std::remove((out + ".env.hdr").c_str());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "harness error: %s\n", e.what());
        return 1;
    }
    return 0;
}
