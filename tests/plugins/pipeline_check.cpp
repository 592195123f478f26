/*
 * A C++ host rendering through the reference's downstream interface on the
 * GPU: livre::RenderPipeline::render(renderParams, redrawFilter,
 * sendHistogramFilter, renderer, availability) with a
 * livre::gb300::CudaRayCastRenderer (a livre::Renderer), the way a Livre
 * channel renders a frame (Channel::Impl::frameDraw, livre/eq/Channel.cpp:
 * 283-336).
 *
 * Usage: pipeline_check <view file> <width> <height> <out.raw>
 * The view file holds float32 values: modelview[16], projection[16] (column
 * major), then 256 RGBA transfer-function entries. The volume is the
 * library's blob volume (128^3 uint8, 32^3 bricks + 1 overlap, 8 blobs,
 * seed 1). Writes the RGBA32F frame (row 0 at the bottom) to out.raw and
 * prints one line per check; exit status 0 when every check holds.
 */
#include <livre/gb300/CudaRayCastRenderer.h>
#include <livre/lib/pipeline/RenderPipeline.h>

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

namespace
{
/* The CUDA renderer with its stage hooks logged. */
class LoggedRenderer : public livre::gb300::CudaRayCastRenderer
{
public:
    using CudaRayCastRenderer::CudaRayCastRenderer;
    std::string log;
    livre::NodeIds ordered;

protected:
    void _onFrameStart(const livre::Frustum& f, const livre::ClipPlanes& p,
                       const livre::PixelViewport& v, const livre::NodeIds& b) override
    {
        log += "start ";
        ordered = b;
        CudaRayCastRenderer::_onFrameStart(f, p, v, b);
    }
    void _onFrameRender(const livre::Frustum& f, const livre::ClipPlanes& p,
                        const livre::PixelViewport& v, const livre::NodeIds& b) override
    {
        log += "render ";
        CudaRayCastRenderer::_onFrameRender(f, p, v, b);
    }
    void _onFrameEnd(const livre::Frustum& f, const livre::ClipPlanes& p,
                     const livre::PixelViewport& v, const livre::NodeIds& b) override
    {
        log += "end";
        CudaRayCastRenderer::_onFrameEnd(f, p, v, b);
    }
};

int bad(const char* what)
{
    std::printf("FAILED %s\n", what);
    return 1;
}
} // namespace

int main(int argc, char** argv)
{
    if (argc != 5)
    {
        std::fprintf(stderr, "usage: %s view width height out.raw\n", argv[0]);
        return 2;
    }
    const uint32_t W = uint32_t(std::atoi(argv[2])), H = uint32_t(std::atoi(argv[3]));
    std::vector<float> view(16 + 16 + 256 * 4);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(view.data(), sizeof(float), view.size(), f) != view.size())
        return bad("reading the view file");
    std::fclose(f);
    try
    {
        lv_ctx* ctx = nullptr;
        livre::gb300::check(lv_ctx_create(0, &ctx), ctx, "lv_ctx_create");
        lv_volume_info info{};
        for (int a = 0; a < 3; ++a)
        {
            info.voxels[a] = 128;
            info.max_block[a] = 34;
            info.overlap[a] = 1;
        }
        info.dtype = LV_DT_UINT8;
        info.comp_count = 1;
        livre::gb300::check(lv_fill_regular_volume_info(&info), ctx, "volume info");
        lv_blob_desc blobs{8, 0, 1};
        lv_volume* vol = nullptr;
        livre::gb300::check(lv_volume_create_blob(ctx, &info, &blobs, LV_BLOB_DEVICE, &vol), ctx,
                            "lv_volume_create_blob");
        lv_tf* tf = nullptr;
        livre::gb300::check(lv_tf_create(ctx, view.data() + 32, 256, &tf), ctx, "lv_tf_create");
        float* d_rgba = nullptr;
        uint8_t* d_rgba8 = nullptr;
        if (cudaMalloc(&d_rgba, size_t(W) * H * 16) != cudaSuccess ||
            cudaMalloc(&d_rgba8, size_t(W) * H * 4) != cudaSuccess)
            return bad("cudaMalloc");

        livre::RenderParams params;
        params.frameInfo = livre::FrameInfo(
            livre::Frustum(livre::Matrix4f(view.data()), livre::Matrix4f(view.data() + 16)), 0, 42);
        params.pixelViewPort = livre::PixelViewport(0, 0, int32_t(W), int32_t(H));
        params.vrParams.setScreenSpaceError(1.0f);
        params.vrParams.setSynchronousMode(true);
        params.vrParams.setLinearFiltering(true);
        params.vrParams.setSamplesPerRay(256);

        uint32_t redraws = 0, histograms = 0, hist_frame = 0;
        uint64_t hist_total = 0;
        livre::PipeFilter redraw([&](const livre::PipeFilterData&) { ++redraws; });
        livre::PipeFilter histogram([&](const livre::PipeFilterData& d) {
            ++histograms;
            hist_frame = d.frameId;
            for (uint32_t b = 0; b < d.nBins; ++b)
                hist_total += d.histogram[b];
        });
        LoggedRenderer renderer(ctx, vol, tf, d_rgba, d_rgba8);
        livre::RenderPipeline pipeline(ctx, vol);
        livre::NodeAvailability availability;
        pipeline.render(params, redraw, histogram, renderer, availability);
        if (cudaDeviceSynchronize() != cudaSuccess)
            return bad("cudaDeviceSynchronize");

        std::vector<float> frame(size_t(W) * H * 4);
        if (cudaMemcpy(frame.data(), d_rgba, frame.size() * 4, cudaMemcpyDeviceToHost) !=
            cudaSuccess)
            return bad("frame copy");
        FILE* o = std::fopen(argv[4], "wb");
        if (!o || std::fwrite(frame.data(), 4, frame.size(), o) != frame.size())
            return bad("writing the frame");
        std::fclose(o);
        const lv_frame_stats& st = renderer.frameStats();
        std::printf("hooks %s\n", renderer.log.c_str());
        std::printf("visible %zu available %zu not_available %zu rendered %u samples %llu "
                    "samples_per_ray %u\n",
                    renderer.ordered.size(), availability.nAvailable, availability.nNotAvailable,
                    st.n_rendered, static_cast<unsigned long long>(st.n_samples),
                    st.samples_per_ray);
        std::printf("filters redraw %u histogram %u frame %u total %llu\n", redraws, histograms,
                    hist_frame, static_cast<unsigned long long>(hist_total));
        std::printf("order");
        for (const livre::NodeId& n : renderer.ordered)
            std::printf(" %llu", static_cast<unsigned long long>(n.getId()));
        std::printf("\n");
        /* interaction: the coarsest allowed level only (maxLOD = minLOD) */
        params.idle = false;
        pipeline.render(params, redraw, histogram, renderer, availability);
        std::printf("interacting visible %zu max_level %u\n", renderer.ordered.size(),
                    renderer.frameStats().max_level);
        cudaFree(d_rgba);
        cudaFree(d_rgba8);
        lv_tf_destroy(tf);
        lv_volume_destroy(vol);
        lv_ctx_destroy(ctx);
    }
    catch (const std::exception& e)
    {
        std::printf("FAILED %s\n", e.what());
        return 1;
    }
    return 0;
}
