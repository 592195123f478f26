/*
 * A C++ host program driving the C ABI the way a Livre channel would
 * (Channel::Impl::frameDraw, livre/eq/Channel.cpp:283-336): load the data
 * source plugins, open a volume by URI, render one view with lv_render,
 * convert it to RGBA8 and write it as a PNG file.
 *
 * Usage: render_check <plugin dir> <uri> <view file> <width> <height> <out.png>
 * The view file holds float32 values: modelview[16], projection[16] (column
 * major), then 256 RGBA transfer-function entries. Prints the frame's
 * statistics; exit status 0 on success.
 */
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>
#include <livre_gb300.h>

namespace
{
int fail(const char* what, lv_ctx* ctx)
{
    std::fprintf(stderr, "%s failed: %s\n", what, ctx ? lv_last_error(ctx) : "");
    return 1;
}
} // namespace

int main(int argc, char** argv)
{
    if (argc != 7)
    {
        std::fprintf(stderr, "usage: %s plugins uri view width height out.png\n", argv[0]);
        return 2;
    }
    const uint32_t W = uint32_t(std::atoi(argv[4])), H = uint32_t(std::atoi(argv[5]));
    std::vector<float> view(16 + 16 + 256 * 4);
    FILE* f = std::fopen(argv[3], "rb");
    if (!f || std::fread(view.data(), sizeof(float), view.size(), f) != view.size())
        return fail("reading the view file", nullptr);
    std::fclose(f);

    uint32_t loaded = 0;
    if (lv_load_plugins(argv[1], nullptr, &loaded) != LV_OK || loaded == 0)
        return fail("lv_load_plugins", nullptr);
    lv_ctx* ctx = nullptr;
    if (lv_ctx_create(0, &ctx) != LV_OK)
        return fail("lv_ctx_create", ctx);
    lv_volume* vol = nullptr;
    if (lv_volume_open(ctx, argv[2], &vol) != LV_OK)
        return fail("lv_volume_open", ctx);
    lv_tf* tf = nullptr;
    if (lv_tf_create(ctx, view.data() + 32, 256, &tf) != LV_OK)
        return fail("lv_tf_create", ctx);

    lv_render_desc d = {};
    for (int i = 0; i < 16; ++i)
    {
        d.camera.modelview[i] = view[i];
        d.camera.projection[i] = view[16 + i];
    }
    d.width = W;
    d.height = H;
    d.lod.window_height = H;
    d.lod.screen_space_error = 1.0f;
    d.lod.min_lod = 0;
    d.lod.max_lod = 100;
    d.lod.range[0] = 0.0f;
    d.lod.range[1] = 1.0f;
    d.step_policy = LV_STEP_HALF_VOXEL;
    d.early_exit = 0.999f;
    d.filter = LV_FILTER_TRILINEAR;
    d.synchronous = 1;
    d.max_uploads = 1;

    float* d_rgba = nullptr;
    if (cudaMalloc(&d_rgba, size_t(W) * H * 16) != cudaSuccess)
        return fail("cudaMalloc", nullptr);
    if (lv_render(ctx, vol, tf, &d, d_rgba, nullptr) != LV_OK)
        return fail("lv_render", ctx);
    lv_frame_stats st;
    if (lv_last_stats(ctx, &st) != LV_OK)
        return fail("lv_last_stats", ctx);
    if (lv_frame_write_png(ctx, d_rgba, W, H, argv[6]) != LV_OK)
        return fail("lv_frame_write_png", ctx);
    std::printf("visible %u rendered %u uploaded %u samples %llu samples_per_ray %u\n",
                st.n_visible, st.n_rendered, st.n_uploaded,
                static_cast<unsigned long long>(st.n_samples), st.samples_per_ray);
    cudaFree(d_rgba);
    lv_tf_destroy(tf);
    lv_volume_destroy(vol);
    lv_ctx_destroy(ctx);
    return 0;
}
