// gb300_renderer.h -- CudaRT's Renderer interface over libcrt_gb300.
//
// A drop-in for ParallelRenderer (src/include/renderer.h:102-126): built in
// the reference's source tree next to its own renderers, constructed by
// main.cpp exactly where ParallelRenderer is (main.cpp:157-164), and driven
// unchanged by TerminalLauncher (terminal_launcher.cpp:10-17) and
// Launcher::saveToImage (launcher.cpp:13-21).  It converts the reference's
// constructed Scene (triangles in BVH order with v1/e1/e2, the deduplicated
// material table with emission already scaled, the light list, textures,
// camera) into a crt_scene_desc, so every input is the reference's own.
#ifndef GB300_RENDERER_H
#define GB300_RENDERER_H

#include "renderer.h"      // the reference's Renderer (src/include/renderer.h)
#include "scene.h"
#include "crt_gb300.h"

class Gb300Renderer : public Renderer {
public:
    // progressive = false (the terminal launcher's case): samples are
    // counted by renderOneSamplePerPixel and rendered together, as one
    // stream of waves, when the image is first read (copyImageBytes).
    // progressive = true: each call renders one sample and writes the
    // formatted image to p_img, like ParallelRenderer.
    __host__ Gb300Renderer(Scene* scene, pixels_t width, pixels_t height, uint samples,
                           bool progressive = false);
    __host__ ~Gb300Renderer();
    __host__ void renderOneSamplePerPixel(uchar4* p_img);
    __host__ void copyImageBytes(uchar4* p_img);
    __host__ uchar4* getImgBytesPointer() { return d_img; }
    __host__ void createMaterialsData() {}   // materials travel with the scene handle

private:
    __host__ void flush();
    crt_scene scene_handle = nullptr;
    crt_render render_handle = nullptr;
    uchar4* d_img = nullptr;
    uint pending = 0;
    bool progressive;
};

#endif
