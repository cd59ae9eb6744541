// Host code of the library under AddressSanitizer and UndefinedBehavior-
// Sanitizer: the scene-file readers (OBJ/MTL, camera JSON, PNG, PNG writer)
// on the files named on the command line, and the host BVH build on seeded
// random and degenerate inputs.  Built and run by tests/test_sanitizers.py;
// no GPU involved (the two library functions that live in CUDA sources are
// stubbed below).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/crt_gb300.h"
#include "../../cudart_gb300/csrc/bvh8.h"

namespace crt {
int set_error(int status, const std::string&) { return status; }
}
extern "C" int crt_camera_from_json(float, float, float, const float*, const float*, const float*, uint32_t w,
                                    uint32_t h, crt_camera* out) {
    std::memset(out, 0, sizeof *out);
    out->xpixels = (int32_t)w;
    out->ypixels = (int32_t)h;
    return CRT_OK;
}

static int run_file(const char* path) {
    const std::string p(path);
    const auto ends = [&](const char* s) { return p.size() >= std::strlen(s) && p.compare(p.size() - std::strlen(s), std::string::npos, s) == 0; };
    if (ends(".obj")) {
        const std::string dir = p.substr(0, p.rfind('/') + 1);
        for (uint32_t flags : {0u, (uint32_t)CRT_LOAD_EXACT_MATERIALS}) {
            crt_scene_files f = nullptr;
            if (crt_scene_files_load(path, dir.c_str(), flags, &f) == CRT_OK) {
                crt_scene_desc d;
                crt_scene_files_desc(f, &d);
                double sum = 0;   // touch every array
                for (uint64_t i = 0; i < 9ull * d.num_triangles; ++i) sum += d.positions[i] + d.normals[i];
                for (uint32_t i = 0; i < d.num_triangles; ++i) sum += d.material_ids[i];
                crt_scene_files_info info;
                crt_scene_files_get_info(f, &info);
                for (uint32_t m = 0; m < info.num_meshes; ++m) {
                    const char* name;
                    uint32_t first, count;
                    crt_scene_files_mesh(f, m, &name, &first, &count);
                    sum += std::strlen(name) + first + count;
                }
                if (std::isnan(sum)) std::printf("nan sum in %s\n", path);
                crt_scene_files_destroy(f);
            }
        }
    } else if (ends(".json")) {
        crt_camera cam;
        crt_camera_load_json(path, 64, 48, &cam);
    } else if (ends(".png")) {
        uint32_t dims[2] = {0, 0};
        if (crt_texture_load_png(path, dims, nullptr, 0) == CRT_OK) {
            std::vector<float> t(3ull * dims[0] * dims[1]);
            crt_texture_load_png(path, dims, t.data(), (uint64_t)dims[0] * dims[1]);
            crt_texture_load_png(path, dims, t.data(), 1);   // too small: an error, no write
        }
    }
    return 0;
}

static void bvh_cases() {
    std::mt19937 rng(7);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    for (uint32_t n : {1u, 2u, 3u, 17u, 1000u, 40000u}) {
        for (int kind = 0; kind < 3; ++kind) {
            std::vector<float> v1(3 * n), e1(3 * n), e2(3 * n);
            for (uint32_t i = 0; i < 3 * n; ++i) {
                v1[i] = kind == 1 ? 0.25f : u(rng);   // kind 1: coincident triangles
                e1[i] = kind == 2 ? 0.f : 0.01f * u(rng);   // kind 2: degenerate (zero-area) triangles
                e2[i] = kind == 2 ? 0.f : 0.01f * u(rng);
            }
            for (int width : {8, 4}) {
                crt::Bvh8 b;
                const char* msg = nullptr;
                if (!crt::build_bvh8(v1.data(), e1.data(), e2.data(), n, 64, b, &msg, width)) {
                    std::printf("build failed n=%u kind=%d: %s\n", n, kind, msg ? msg : "?");
                    std::exit(2);
                }
                if (b.tris.size() != n) {
                    std::printf("lost triangles n=%u kind=%d\n", n, kind);
                    std::exit(2);
                }
            }
        }
    }
}

int main(int argc, char** argv) {
    for (int i = 1; i < argc; ++i) run_file(argv[i]);
    if (argc == 1) bvh_cases();
    std::printf("sanitize_host: ok\n");
    return 0;
}
