// nanogi command line: the interface of src/nanogi.cpp:1993-2151 on the GB300 renderer.
//
//   nanogi [options] <renderer> <scene> <result> <width> <height>
//
// Same option names, short forms, defaults and positional order as the reference
// (src/nanogi.cpp:2000-2023). Options that steer the reference's CPU thread pool
// (--num-threads, --grain-size, --progress-update-interval) are accepted and have no
// effect on the GPU. GPU-only options: --seed, --precision, --raster, --wave-size.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <map>
#include <string>
#include <vector>

#include "../../include/nanogi.h"

namespace {

struct Opt {
    std::string value;
    bool set = false;
};

void Usage() {
    std::printf(
        "Usage: nanogi [options] <renderer> <scene> <result> <width> <height>\n"
        "Allowed options:\n"
        "  --help                               Display help message\n"
        "  -i [ --scene ] arg                   Scene file\n"
        "  -o [ --result ] arg (=render.hdr)    Rendered result (.hdr or .pfm)\n"
        "  -r [ --renderer ] arg                Rendering technique (pt, ptdirect)\n"
        "  -n [ --num-samples ] arg (=10000000) Number of samples\n"
        "  -m [ --max-num-vertices ] arg (=-1)  Maximum number of vertices\n"
        "  -w [ --width ] arg (=1280)           Width of the rendered image\n"
        "  -h [ --height ] arg (=720)           Height of the rendered image\n"
        "  -j [ --num-threads ] arg             Number of threads (no effect on the GPU)\n"
        "  --grain-size arg (=10000)            Grain size (no effect on the GPU)\n"
        "  --progress-update-interval arg (=100000)\n"
        "  -t [ --render-time ] arg (=-1)       Render time in seconds (-1 to use # of samples)\n"
        "  --progress-image-update-interval arg (=-1)\n"
        "  --progress-image-update-format arg (=progress/{{count}}.png)\n"
        "  --seed arg (=time)                   Philox seed (paths are replayable per seed)\n"
        "  --precision arg (=fp32)              fp32 (tuned) or fp64 (plain) shading\n"
        "  --raster arg (=stratified)           stratified or uniform camera samples\n"
        "  --wave-size arg (=0)                 path slots on the device (0 = auto)\n");
}

}  // namespace

int main(int argc, char** argv) {
    if (argc == 1) {
        Usage();
        return EXIT_FAILURE;
    }
    const std::map<std::string, std::string> shorts = {{"-i", "scene"}, {"-o", "result"}, {"-r", "renderer"},
                                                       {"-n", "num-samples"}, {"-m", "max-num-vertices"},
                                                       {"-w", "width"}, {"-h", "height"}, {"-j", "num-threads"},
                                                       {"-t", "render-time"}};
    const std::vector<std::string> longs = {"scene", "result", "renderer", "num-samples", "max-num-vertices", "width",
                                            "height", "num-threads", "grain-size", "progress-update-interval",
                                            "render-time", "progress-image-update-interval",
                                            "progress-image-update-format", "seed", "precision", "raster",
                                            "wave-size"};
    std::map<std::string, Opt> o;
    o["result"].value = "render.hdr";
    o["num-samples"].value = "10000000";
    o["max-num-vertices"].value = "-1";
    o["width"].value = "1280";
    o["height"].value = "720";
    o["render-time"].value = "-1";
    o["precision"].value = "fp32";
    o["raster"].value = "stratified";
    o["wave-size"].value = "0";
    const std::vector<std::string> positional = {"renderer", "scene", "result", "width", "height"};
    size_t pos_i = 0;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "--help") {
            Usage();
            return EXIT_FAILURE;
        }
        std::string key;
        std::string val;
        bool has_val = false;
        if (a.rfind("--", 0) == 0) {
            key = a.substr(2);
            const size_t eq = key.find('=');
            if (eq != std::string::npos) {
                val = key.substr(eq + 1);
                key = key.substr(0, eq);
                has_val = true;
            }
            bool known = false;
            for (auto& l : longs) known |= l == key;
            if (!known) {
                std::fprintf(stderr, "ERROR : unrecognised option '%s'\n", a.c_str());
                return EXIT_FAILURE;
            }
        } else if (a.size() >= 2 && a[0] == '-' && shorts.count(a.substr(0, 2))) {
            key = shorts.at(a.substr(0, 2));
            if (a.size() > 2) {
                val = a.substr(2);
                has_val = true;
            }
        } else {
            if (pos_i >= positional.size()) {
                std::fprintf(stderr, "ERROR : too many positional options\n");
                return EXIT_FAILURE;
            }
            o[positional[pos_i]].value = a;
            o[positional[pos_i]].set = true;
            pos_i++;
            continue;
        }
        if (!has_val) {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "ERROR : the required argument for option '--%s' is missing\n", key.c_str());
                return EXIT_FAILURE;
            }
            val = argv[++i];
        }
        o[key].value = val;
        o[key].set = true;
    }
    if (!o["renderer"].set) {
        std::fprintf(stderr, "ERROR : the option '--renderer' is required but missing\n");
        return EXIT_FAILURE;
    }
    if (!o["scene"].set) {
        std::fprintf(stderr, "ERROR : the option '--scene' is required but missing\n");
        return EXIT_FAILURE;
    }
    ngi_render_params p;
    std::memset(&p, 0, sizeof(p));
    const std::string r = o["renderer"].value;
    if (r == "pt") p.renderer = NGI_RENDERER_PT;
    else if (r == "ptdirect") p.renderer = NGI_RENDERER_PTDIRECT;
    else if (r == "lt") p.renderer = NGI_RENDERER_LT;
    else if (r == "ltdirect") p.renderer = NGI_RENDERER_LTDIRECT;
    else if (r == "bdpt") p.renderer = NGI_RENDERER_BDPT;
    else {
        std::fprintf(stderr, "ERROR : renderer '%s' is not built (available: pt, ptdirect, lt, ltdirect, bdpt)\n",
                     r.c_str());
        return EXIT_FAILURE;
    }
    try {
        p.num_samples = std::stoll(o["num-samples"].value);
        p.max_num_vertices = std::stoi(o["max-num-vertices"].value);
        p.width = std::stoi(o["width"].value);
        p.height = std::stoi(o["height"].value);
        p.wave_size = std::stoi(o["wave-size"].value);
        p.seed = o["seed"].set ? std::stoull(o["seed"].value) : (unsigned long long)std::time(nullptr);
    } catch (const std::exception&) {
        std::fprintf(stderr, "ERROR : invalid numeric option\n");
        return EXIT_FAILURE;
    }
    const std::string prec = o["precision"].value;
    if (prec == "fp32") p.precision = NGI_PRECISION_FP32;
    else if (prec == "fp64") p.precision = NGI_PRECISION_FP64;
    else {
        std::fprintf(stderr, "ERROR : --precision must be fp32 or fp64\n");
        return EXIT_FAILURE;
    }
    const std::string ras = o["raster"].value;
    if (ras == "stratified") p.raster_mode = NGI_RASTER_STRATIFIED;
    else if (ras == "uniform") p.raster_mode = NGI_RASTER_UNIFORM;
    else {
        std::fprintf(stderr, "ERROR : --raster must be stratified or uniform\n");
        return EXIT_FAILURE;
    }
    if (p.width <= 0 || p.height <= 0) {
        std::fprintf(stderr, "ERROR : width and height must be positive\n");
        return EXIT_FAILURE;
    }
    const double render_time = std::atof(o["render-time"].value.c_str());
    const double image_interval = std::atof(o["progress-image-update-interval"].value.c_str());
    const std::string image_format = o["progress-image-update-format"].value;

    std::fprintf(stderr, "nanogi-gb300\nLoading scene\n");
    ngi_scene* scene = nullptr;
    if (ngi_scene_load(o["scene"].value.c_str(), (double)p.width / p.height, &scene) != NGI_OK) {
        std::fprintf(stderr, "ERROR : %s\n", ngi_last_error());
        return EXIT_FAILURE;
    }
    std::vector<double> film(3 * (size_t)p.width * p.height, 0.0);
    std::fprintf(stderr, "Rendering\n");
    const auto t0 = std::chrono::steady_clock::now();
    ngi_status st = NGI_OK;
    long long processed = 0;
    // Progress images (src/nanogi.cpp:356-404): after a batch of samples, when more than the
    // interval has passed since the last one, the film so far goes to the format path with
    // {{count}} replaced by the image count as %010d.
    long long image_count = 0;
    auto last_image = t0;
    auto progress_image = [&](const std::vector<double>& f) {
        if (!(image_interval > 0)) return;
        const auto now = std::chrono::steady_clock::now();
        if (std::chrono::duration<double>(now - last_image).count() <= image_interval) return;
        char count[32];
        std::snprintf(count, sizeof(count), "%010lld", ++image_count);
        std::string path = image_format;
        for (size_t at = path.find("{{count}}"); at != std::string::npos; at = path.find("{{count}}", at))
            path.replace(at, 9, count);
        std::fprintf(stderr, "Saving progress: %s\n", path.c_str());
        if (ngi_save_image(path.c_str(), f.data(), p.width, p.height) != NGI_OK)
            std::fprintf(stderr, "ERROR : %s\n", ngi_last_error());
        last_image = now;
    };
    if (render_time < 0) {
        st = ngi_render(scene, &p, film.data());
        processed = p.num_samples;
        if (st == NGI_OK) progress_image(film);
    } else {
        // Time-budget mode (src/nanogi.cpp:243, 326-334): whole-image passes until time is up.
        std::vector<double> part(film.size()), sum(film.size(), 0.0);
        ngi_render_params q = p;
        q.num_samples = (long long)p.width * p.height;
        while (st == NGI_OK) {
            q.sample_offset = processed;
            st = ngi_render(scene, &q, part.data());
            if (st != NGI_OK) break;
            processed += q.num_samples;
            // part is normalised per pass; accumulate un-normalised sums
            for (size_t k = 0; k < sum.size(); k++) sum[k] += part[k];
            const double passes = (double)processed / q.num_samples;
            for (size_t k = 0; k < film.size(); k++) film[k] = sum[k] / passes;
            progress_image(film);
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (el > render_time) break;
        }
    }
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st != NGI_OK) {
        std::fprintf(stderr, "ERROR : %s\n", ngi_last_error());
        ngi_scene_free(scene);
        return EXIT_FAILURE;
    }
    ngi_render_stats stats;
    ngi_get_render_stats(scene, &stats);
    std::fprintf(stderr, "# of samples: %lld\nElapesed time: %.3f\n", processed, el);
    std::fprintf(stderr, "Rays: camera %lld extension %lld shadow %lld\n", (long long)stats.camera_rays,
                 (long long)stats.extension_rays, (long long)stats.shadow_rays);
    std::fprintf(stderr, "Saving rendered image\n");
    if (ngi_save_image(o["result"].value.c_str(), film.data(), p.width, p.height) != NGI_OK) {
        std::fprintf(stderr, "ERROR : %s\n", ngi_last_error());
        ngi_scene_free(scene);
        return EXIT_FAILURE;
    }
    ngi_scene_free(scene);
    return EXIT_SUCCESS;
}
