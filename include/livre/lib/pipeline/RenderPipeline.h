/*
 * livre::RenderPipeline on the GPU: the per-frame pipeline of
 * livre/lib/pipeline/RenderPipeline.h:39-85 (RenderParams, render) over this
 * library's C ABI. Header only.
 *
 * RenderPipeline::render(renderParams, redrawFilter, sendHistogramFilter,
 * renderer, availability) keeps the reference's signature and steps
 * (RenderPipeline.cpp:60-158, 268-278):
 *  - the visible set of the view on the device (lv_select_visible_host: the
 *    VisibleSetGeneratorFilter's "VisibleNodes"), with the reference's
 *    coarsest-LOD clamp while the user interacts (idle false: maxLOD =
 *    minLOD, RenderPipeline.cpp:71-74);
 *  - renderer.render(frustum, clipPlanes, pixelViewport, visible, RENDER_ALL):
 *    order() and the stage hooks. A renderer that also derives from
 *    gb300::DeviceFrameRenderer (gb300::CudaRayCastRenderer) first receives
 *    the frame's lv_render_desc and renders the whole frame with lv_render
 *    in its RENDER_FRAME hook: residency (synchronous or asynchronous as
 *    vrParams.getSynchronousMode() says) and the ray cast, in pool-sized
 *    passes when the visible set exceeds the brick pool;
 *  - availability: the frame's available / not available bricks;
 *  - sendHistogramFilter: the frame's value histogram (lv_frame_histogram,
 *    HistogramFilter.cpp:78-149), with the frame id and relative viewport;
 *  - redrawFilter: executed when bricks were not available (asynchronous
 *    mode), so the application renders again, as the reference's upload
 *    filter triggers a redraw when data arrives.
 * The reference's data and texture caches and its texture pool are the
 * context's HBM brick pool (lv_pool_configure); its GL context is the
 * context's CUDA device. Errors throw std::runtime_error with
 * lv_last_error's message (the reference throws, LBTHROW).
 */
#ifndef LIVRE_GB300_COMPAT_RENDERPIPELINE_H
#define LIVRE_GB300_COMPAT_RENDERPIPELINE_H

#include <livre/core/render/FrameInfo.h>
#include <livre/core/render/Renderer.h>
#include <livre/lib/configuration/VolumeRendererParameters.h>
#include <livre_gb300.h>

#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

namespace livre
{
/* Parameters of one frame (RenderPipeline.h:39-49). */
struct RenderParams
{
    VolumeRendererParameters vrParams;
    FrameInfo frameInfo;
    Range renderDataRange{{0.0f, 1.0f}};
    Vector2f dataSourceRange{0.0f, 0.0f};
    PixelViewport pixelViewPort;
    Viewport viewport{0.0f, 0.0f, 1.0f, 1.0f};
    ClipPlanes clipPlanes;
    bool idle = true;
};

/* What a pipeline filter receives after a frame. */
struct PipeFilterData
{
    uint32_t frameId = 0;
    Viewport viewport;
    NodeAvailability availability;
    const uint64_t* histogram = nullptr; /* nBins counts (sendHistogramFilter) */
    uint32_t nBins = 0;
    float histogramRange[2] = {0.0f, 0.0f};
};

/* A filter of the reference's pipeline (PipeFilter), as the callable the
 * render pipeline executes. */
class PipeFilter
{
public:
    typedef std::function<void(const PipeFilterData&)> Function;
    PipeFilter() = default;
    explicit PipeFilter(Function fn) : _fn(std::move(fn)) {}
    void execute(const PipeFilterData& data) const
    {
        if (_fn)
            _fn(data);
    }
    explicit operator bool() const { return bool(_fn); }

private:
    Function _fn;
};

namespace gb300
{
inline void check(lv_status st, lv_ctx* ctx, const char* what)
{
    if (st != LV_OK)
        throw std::runtime_error(std::string(what) + ": " + (ctx ? lv_last_error(ctx) : ""));
}

/* The lv_render_desc of one frame (RenderPipeline.cpp:60-90 and
 * RayCastRenderer.cpp:213-386): camera, viewport, LOD parameters (with the
 * interaction clamp), samples per ray (0: the reference's rule), filtering
 * (linear_filtering: trilinear, else nearest), data range, residency mode. */
inline lv_render_desc makeRenderDesc(const RenderParams& p)
{
    lv_render_desc d{};
    const Frustum& f = p.frameInfo.frustum;
    for (int i = 0; i < 16; ++i)
    {
        d.camera.modelview[i] = f.getMVMatrix().array[i];
        d.camera.projection[i] = f.getProjMatrix().array[i];
    }
    d.width = uint32_t(p.pixelViewPort[2]);
    d.height = uint32_t(p.pixelViewPort[3]);
    d.lod.window_height = d.height;
    d.lod.screen_space_error = p.vrParams.getScreenSpaceError();
    d.lod.min_lod = p.vrParams.getMinLod();
    d.lod.max_lod = p.idle ? p.vrParams.getMaxLod() : p.vrParams.getMinLod();
    d.lod.range[0] = p.renderDataRange[0];
    d.lod.range[1] = p.renderDataRange[1];
    d.lod.time_step = p.frameInfo.timeStep;
    const std::vector<ClipPlane>& planes = p.clipPlanes.getPlanes();
    if (planes.size() > 6)
        throw std::runtime_error("more than 6 clip planes");
    d.lod.n_clip_planes = uint32_t(planes.size());
    for (size_t i = 0; i < planes.size(); ++i)
    {
        for (int k = 0; k < 3; ++k)
            d.lod.clip_planes[i][k] = planes[i].getNormal()[k];
        d.lod.clip_planes[i][3] = planes[i].getD();
    }
    d.samples_per_ray = p.vrParams.getSamplesPerRay();
    d.step_policy = LV_STEP_REFERENCE;
    d.early_exit = 0.999f;
    d.filter = p.vrParams.getLinearFiltering() ? LV_FILTER_TRILINEAR : LV_FILTER_NEAREST;
    d.data_range[0] = p.dataSourceRange[0];
    d.data_range[1] = p.dataSourceRange[1];
    d.synchronous = p.vrParams.getSynchronousMode() ? 1u : 0u;
    d.max_uploads = 1;
    return d;
}

/* A renderer that draws a whole frame on the device: it takes the frame's
 * description before render() and reports the frame's statistics after. */
class DeviceFrameRenderer
{
public:
    virtual void setRenderDesc(const lv_render_desc& desc) = 0;
    virtual const lv_frame_stats& frameStats() const = 0;
    virtual ~DeviceFrameRenderer() {}
};
} // namespace gb300

class RenderPipeline
{
public:
    /* ctx: the context (brick pool, device); volume: the volume the frames
     * render (lv_volume_open of a data source URI, or any lv_volume_*). */
    RenderPipeline(lv_ctx* ctx, lv_volume* volume) : _ctx(ctx), _volume(volume)
    {
        gb300::check(lv_volume_get_info(volume, &_info), ctx, "lv_volume_get_info");
    }

    void render(const RenderParams& renderParams, PipeFilter redrawFilter,
                PipeFilter sendHistogramFilter, Renderer& renderer,
                NodeAvailability& availability) const
    {
        const lv_render_desc desc = gb300::makeRenderDesc(renderParams);
        /* the visible set, as the visible-set generator filter delivers it */
        uint32_t res[LV_SELECT_RESULT_WORDS] = {};
        std::vector<uint64_t> ids(1024);
        for (;;)
        {
            gb300::check(lv_select_visible_host(_ctx, &_info, &desc.camera, &desc.lod,
                                                ids.data(), uint32_t(ids.size()), res),
                         _ctx, "lv_select_visible_host");
            if (res[LV_SEL_FOUND] <= ids.size())
                break;
            ids.resize(res[LV_SEL_FOUND]);
        }
        NodeIds visible;
        visible.reserve(res[LV_SEL_WRITTEN]);
        for (uint32_t i = 0; i < res[LV_SEL_WRITTEN]; ++i)
            visible.push_back(NodeId(ids[i]));

        gb300::DeviceFrameRenderer* device = dynamic_cast<gb300::DeviceFrameRenderer*>(&renderer);
        if (device)
            device->setRenderDesc(desc);
        renderer.render(renderParams.frameInfo.frustum, renderParams.clipPlanes,
                        renderParams.pixelViewPort, visible, RENDER_ALL);

        PipeFilterData data;
        data.frameId = renderParams.frameInfo.frameId;
        data.viewport = renderParams.viewport;
        if (device)
        {
            availability.nAvailable = device->frameStats().n_available;
            availability.nNotAvailable = device->frameStats().n_not_available;
        }
        else
        {
            availability.nAvailable = visible.size();
            availability.nNotAvailable = 0;
        }
        data.availability = availability;
        if (sendHistogramFilter && device)
        {
            std::vector<uint64_t> hist(256);
            float lo = 0.0f, hi = 0.0f;
            typeRange(lo, hi);
            if (desc.data_range[1] > 0.0f && desc.data_range[1] > desc.data_range[0])
            {
                lo = desc.data_range[0];
                hi = desc.data_range[1];
            }
            gb300::check(lv_frame_histogram(_ctx, 256, lo, hi, hist.data()), _ctx,
                         "lv_frame_histogram");
            data.histogram = hist.data();
            data.nBins = 256;
            data.histogramRange[0] = lo;
            data.histogramRange[1] = hi;
            sendHistogramFilter.execute(data);
            data.histogram = nullptr;
            data.nBins = 0;
        }
        if (availability.nNotAvailable > 0)
            redrawFilter.execute(data);
    }

    const lv_volume_info& getVolumeInfo() const { return _info; }

private:
    /* the value range of the volume's voxel type (RayCastRenderer.cpp:236-277) */
    void typeRange(float& lo, float& hi) const
    {
        switch (_info.dtype)
        {
        case LV_DT_UINT8: lo = 0.0f; hi = 255.0f; break;
        case LV_DT_UINT16: lo = 0.0f; hi = 65535.0f; break;
        case LV_DT_INT8: lo = -128.0f; hi = 127.0f; break;
        case LV_DT_INT16: lo = -32768.0f; hi = 32767.0f; break;
        case LV_DT_UINT32: lo = 0.0f; hi = 4294967295.0f; break;
        case LV_DT_INT32: lo = -2147483648.0f; hi = 2147483647.0f; break;
        default: lo = 1.17549435e-38f; hi = 3.40282347e+38f; break; /* float */
        }
    }

    lv_ctx* _ctx;
    lv_volume* _volume;
    lv_volume_info _info{};
};
} // namespace livre

#endif
