// crt_render -- command-line renderer over the library's C ABI.
//
// Same options, scene lookup and output as the reference's CudaRT binary
// (src/main.cpp:24-188): `-f <scene>` reads <meshes>/<scene>.obj and
// <settings>/<scene>-camera.json with textures from <textures>/, the three
// folders taken from ../.env (MESHES_PATH, CAMERA_PATH, TEXTURES_PATH;
// src/context/env_loader.cpp:14-37) or ../meshes, ../settings, ../textures;
// `-s` samples per pixel (10), `-w`/`-h` image size (640 x 480); the image is
// written to <scene>.png (out.png without -f) after the timed render +
// resolve, as TerminalLauncher and Launcher::saveToImage do
// (terminal_launcher.cpp:10-17, launcher.cpp:13-21).
//
// Additions: -o <file> (advertised by the reference, never parsed there),
// --mode wavefront|megakernel, --depth N (the reference's 6 bounces by
// default), --seed N, --builder host|gpu, --nodes f32|q8 (node encoding the
// render reads; FP32 by default), --tune (autotune the wavefront
// options first), --exact-materials, --env <file>, --json (one JSON line of
// timings).  --cpu and --x have no counterpart here: this renderer runs on
// the GPU only and has no window.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/crt_gb300.h"

namespace {

struct Failure {
    std::string what;
};

void check(int status, const char* call) {
    if (status != CRT_OK) throw Failure{std::string(call) + ": " + crt_last_error()};
}

// Value of `flag` as the reference reads it: the first occurrence, when it
// is not the last argument.
bool flag_value(const std::vector<std::string>& args, const std::string& flag, std::string& out) {
    for (size_t i = 0; i < args.size(); ++i)
        if (args[i] == flag) {
            if (i + 1 >= args.size()) return false;
            out = args[i + 1];
            return true;
        }
    return false;
}

bool has_flag(const std::vector<std::string>& args, const std::string& flag) {
    for (const auto& a : args)
        if (a == flag) return true;
    return false;
}

void int_option(const std::vector<std::string>& args, const char* flag, int& value) {
    std::string v;
    if (!flag_value(args, flag, v)) return;
    try {
        value = std::stoi(v);
    } catch (const std::exception&) {
        std::cerr << "Invalid argument to " << flag << "!" << std::endl;
    }
}

// KEY=value lines; '#' comments.
std::map<std::string, std::string> read_env(const std::string& path, bool& found) {
    std::map<std::string, std::string> kv;
    std::ifstream f(path);
    found = f.is_open();
    std::string line;
    while (found && std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.empty() || line[0] == '#') continue;
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        kv[line.substr(0, eq)] = line.substr(eq + 1);
    }
    return kv;
}

void usage() {
    std::cerr << "Usage: crt_render <options>\n"
                 "-o \t<output file>\tdefault: <scene>.png\n"
                 "-s \t<number of samples>\tdefault:10\n"
                 "-w \t<width>\tdefault:640px\n"
                 "-h \t<height>\tdefault:480px\n"
                 "-f \t<scene>\tdefault: cornell\n"
                 "--mode \t<wavefront|megakernel>\tdefault: wavefront\n"
                 "--depth \t<max bounces>\tdefault: 6\n"
                 "--seed \t<Philox seed>\tdefault: 1234\n"
                 "--builder \t<host|gpu>\tdefault: host\n"
                 "--nodes \t<f32|q8>\tdefault: f32\n"
                 "--tune \t<autotune the wavefront options first>\n"
                 "--exact-materials \t<one material per MTL entry>\n"
                 "--env \t<.env file>\tdefault: ../.env\n"
                 "--json \t<print a JSON line of timings>\n";
}

int run(int argc, char** argv) {
    int samples = 10, width = 640, height = 480, depth = 6, seed = 1234;
    std::string out_file = "out.png", scene_name = "cornell";
    std::vector<std::string> args(argv + 1, argv + argc);
    if (args.empty()) {
        usage();
        return 1;
    }
    if (has_flag(args, "--cpu")) {
        std::cerr << "--cpu: this renderer has no CPU path (it renders on the GPU only)" << std::endl;
        return 2;
    }
    if (has_flag(args, "--x")) {
        std::cerr << "--x: this renderer has no window; the image is written to a PNG file" << std::endl;
        return 2;
    }
    std::string env_path = "../.env";
    flag_value(args, "--env", env_path);
    bool env_found = false;
    auto env = read_env(env_path, env_found);
    auto dir = [&](const char* key, const char* fallback) {
        auto it = env.find(key);
        return (env_found && it != env.end() ? it->second : std::string(fallback)) + "/";
    };
    const std::string obj_dir = dir("MESHES_PATH", "../meshes"), cam_dir = dir("CAMERA_PATH", "../settings"),
                      tex_dir = dir("TEXTURES_PATH", "../textures");
    int_option(args, "-s", samples);
    int_option(args, "-w", width);
    int_option(args, "-h", height);
    int_option(args, "--depth", depth);
    int_option(args, "--seed", seed);
    std::string v;
    if (flag_value(args, "-f", v)) {
        scene_name = v;
        out_file = scene_name + ".png";
    }
    if (flag_value(args, "-o", v)) out_file = v;
    const std::string obj_path = obj_dir + scene_name + ".obj";
    const std::string cam_path = cam_dir + scene_name + "-camera.json";
    std::string mode = "wavefront", builder = "host", nodes = "f32";
    flag_value(args, "--mode", mode);
    flag_value(args, "--builder", builder);
    flag_value(args, "--nodes", nodes);
    if (mode != "wavefront" && mode != "megakernel") throw Failure{"--mode must be wavefront or megakernel"};
    if (builder != "host" && builder != "gpu") throw Failure{"--builder must be host or gpu"};
    if (nodes != "f32" && nodes != "q8") throw Failure{"--nodes must be f32 or q8"};
    if (samples < 1 || width < 1 || height < 1 || depth < 1) throw Failure{"-s, -w, -h and --depth must be positive"};
    const bool json = has_flag(args, "--json");

    std::cout << "Samples: " << samples << std::endl
              << "Width: " << width << std::endl
              << "Height: " << height << std::endl
              << "Obj path: " << obj_path << std::endl
              << "Camera path: " << cam_path << std::endl
              << "Output: " << out_file << std::endl;

    using Clock = std::chrono::steady_clock;
    const auto t_load = Clock::now();
    crt_scene_files files = nullptr;
    check(crt_scene_files_load(obj_path.c_str(), tex_dir.c_str(),
                               has_flag(args, "--exact-materials") ? CRT_LOAD_EXACT_MATERIALS : 0u, &files),
          "loading the scene files");
    crt_scene_files_info finfo;
    check(crt_scene_files_get_info(files, &finfo), "crt_scene_files_get_info");
    crt_camera camera;
    check(crt_camera_load_json(cam_path.c_str(), (uint32_t)width, (uint32_t)height, &camera), "loading the camera");
    for (uint32_t m = 0; m < finfo.num_meshes && m < 64; ++m) {
        const char* name = nullptr;
        uint32_t first = 0, count = 0;
        check(crt_scene_files_mesh(files, m, &name, &first, &count), "crt_scene_files_mesh");
        std::cout << "Mesh " << m << ": `" << name << "`" << std::endl
                  << "\t" << 3 * count << " vertices | \t" << count << " triangles" << std::endl;
    }
    if (finfo.num_meshes > 64) std::cout << "(" << finfo.num_meshes - 64 << " more meshes)" << std::endl;
    std::cout << "Total number of triangles:\t" << finfo.num_triangles << std::endl;

    crt_scene_desc desc;
    check(crt_scene_files_desc(files, &desc), "crt_scene_files_desc");
    desc.builder = builder == "gpu" ? CRT_BVH_GPU : CRT_BVH_HOST;
    crt_scene scene = nullptr;
    check(crt_scene_create(&desc, &scene), "crt_scene_create");
    crt_scene_files_destroy(files);
    const double load_s = std::chrono::duration<double>(Clock::now() - t_load).count();

    crt_render_options opts;
    crt_render_options_default(&opts);
    opts.mode = mode == "wavefront" ? CRT_MODE_WAVEFRONT : CRT_MODE_MEGAKERNEL;
    opts.max_depth = (uint32_t)depth;
    opts.seed = (uint64_t)seed;
    opts.node_format = nodes == "f32" ? CRT_NODES_F32 : CRT_NODES_Q8;
    if (has_flag(args, "--tune")) {
        if (mode != "wavefront") throw Failure{"--tune applies to the wavefront mode"};
        crt_tune_params params;
        crt_tune_params_default(&params);
        crt_tune_result res;
        check(crt_autotune(scene, &camera, (uint32_t)width, (uint32_t)height, &opts, &params, &res), "crt_autotune");
        opts = res.options;
        std::cout << "Autotuned " << res.candidates << " candidates in " << res.tune_ms / 1000.0f
                  << " s: " << res.start_ms_per_spp << " -> " << res.ms_per_spp << " ms per sample" << std::endl;
    }
    crt_render r = nullptr;
    check(crt_render_create(scene, &camera, (uint32_t)width, (uint32_t)height, &opts, &r), "crt_render_create");
    std::cout << "\nLaunching crt_render (GB300, C ABI " << crt_api_version() << ", " << mode << ")" << std::endl;

    std::vector<uint8_t> rgba((size_t)width * height * 4);
    const auto t0 = Clock::now();
    check(crt_render_pass(r, (uint32_t)samples), "crt_render_pass");
    check(crt_render_resolve(r, rgba.data()), "crt_render_resolve");
    const double elapsed = std::chrono::duration<double>(Clock::now() - t0).count();
    uint32_t rendered = 0;
    check(crt_render_samples_rendered(r, &rendered), "crt_render_samples_rendered");
    check(crt_image_write_png(out_file.c_str(), (uint32_t)width, (uint32_t)height, rgba.data()), "writing the image");
    crt_render_destroy(r);
    crt_scene_destroy(scene);

    std::cout << "Rendered to " << out_file << " for " << rendered << " samples per pixel. " << std::endl;
    std::cout << "Elapsed time in seconds = " << elapsed << std::endl;
    std::cout << "Average samples per pixel = " << rendered / elapsed << std::endl;
    const double msps = (double)width * height * rendered / elapsed / 1e6;
    std::cout << "Msamples/s = " << msps << std::endl;
    if (json) {
        char line[512];
        std::snprintf(line, sizeof line,
                      "{\"scene\": \"%s\", \"triangles\": %u, \"width\": %d, \"height\": %d, \"spp\": %u, "
                      "\"mode\": \"%s\", \"load_s\": %.4f, \"parse_ms\": %.2f, \"render_s\": %.4f, "
                      "\"msamples_per_s\": %.2f}",
                      scene_name.c_str(), finfo.num_triangles, width, height, rendered,
                      mode.c_str(), load_s, finfo.parse_ms, elapsed, msps);
        std::cout << line << std::endl;
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        return run(argc, argv);
    } catch (const Failure& f) {
        std::cerr << "crt_render: " << f.what << std::endl;
        return 1;
    }
}
