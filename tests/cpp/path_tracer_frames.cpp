// Headless frames through the C++ PathTracer interface (include/xr_path_tracer.hpp):
//   path_tracer_frames <width> <height> <frames> <out.rgba8> [compat]
// renders the Cornell box for <frames> DrawFrame() calls and writes the last frame's
// tone-mapped RGBA8 image.  The GPU tests compare it with the Python PathTracer.
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <vector>

#include "xr_path_tracer.hpp"

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s width height frames out.rgba8 [compat]\n", argv[0]);
        return 2;
    }
    const uint32_t w = (uint32_t)std::atoi(argv[1]), h = (uint32_t)std::atoi(argv[2]);
    const int frames = std::atoi(argv[3]);
    try {
        xr::UserSettings s;
        s.compat_reference = argc > 5 && std::atoi(argv[5]) != 0;
        xr::PathTracer pt(s, w, h);
        pt.PostTracerInit({xr::HostScene::Cornell()});
        for (int f = 0; f < frames; f++) pt.DrawFrame();
        std::vector<uint32_t> rgba((size_t)w * h);
        pt.ReadOutput(XR_OUT_LDR8, rgba);
        std::FILE* out = std::fopen(argv[4], "wb");
        if (!out || std::fwrite(rgba.data(), 4, rgba.size(), out) != rgba.size()) {
            std::fprintf(stderr, "cannot write %s\n", argv[4]);
            return 1;
        }
        std::fclose(out);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
