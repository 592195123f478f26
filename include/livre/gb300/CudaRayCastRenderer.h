/*
 * livre::gb300::CudaRayCastRenderer: the ray-cast renderer of
 * livre/eq/render/RayCastRenderer.{h,cpp} as a livre::Renderer subclass over
 * this library's C ABI. Header only.
 *
 *  - order(): the bricks sorted by the eye-space distance of their world-box
 *    centres, nearest first (RayCastRenderer.cpp:57-81, 153-159); ties keep
 *    their input order.
 *  - _onFrameStart: the frame's lv_render_desc; without a render pipeline
 *    (setRenderDesc not called) one is made from the frustum, clip planes
 *    and pixel viewport with the defaults of VolumeRendererParameters
 *    (RayCastRenderer.cpp:213-386 uploads the same uniforms).
 *  - _onFrameRender: lv_render of the frame into the RGBA32F device target
 *    (the reference's render texture): LOD selection, residency and the ray
 *    cast of every visible brick in per-ray order.
 *  - _onFrameEnd: the RGBA8 copy of the frame (fragTexCopy.glsl:11-15,
 *    RayCastRenderer.cpp:618-638) into an optional device buffer.
 * Failures throw std::runtime_error with lv_last_error's message.
 */
#ifndef LIVRE_GB300_CUDARAYCASTRENDERER_H
#define LIVRE_GB300_CUDARAYCASTRENDERER_H

#include <livre/core/render/Renderer.h>
#include <livre/lib/pipeline/RenderPipeline.h>
#include <livre_gb300.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace livre
{
namespace gb300
{
/* World box of a node (DataSourcePlugin.cpp:40-71): position / bricks of
 * the level's largest axis, times the world size, centred. */
inline Boxf nodeWorldBox(const lv_volume_info& info, const NodeId& node)
{
    const uint32_t L = node.getLevel();
    const uint32_t b[3] = {info.root_blocks[0] << L, info.root_blocks[1] << L,
                           info.root_blocks[2] << L};
    size_t m = 0;
    for (size_t i = 1; i < 3; ++i)
        if (b[i] > b[m])
            m = i;
    const float denom = float(b[m]);
    const Vector3ui p = node.getPosition();
    Vector3f lo, hi;
    for (size_t i = 0; i < 3; ++i)
    {
        const float ws = info.world_size[i];
        lo[i] = float(p[i]) / denom * ws - ws * 0.5f;
        hi[i] = float(p[i] + 1u) / denom * ws - ws * 0.5f;
    }
    return Boxf(lo, hi);
}

/* The reference's brick order: ascending |modelview * box centre|. */
inline NodeIds distanceOrder(const NodeIds& bricks, const Frustum& frustum,
                             const lv_volume_info& info)
{
    const Matrix4f& mv = frustum.getMVMatrix();
    std::vector<float> dist(bricks.size());
    for (size_t n = 0; n < bricks.size(); ++n)
    {
        const Vector3f c = nodeWorldBox(info, bricks[n]).getCenter();
        float e[3];
        for (size_t r = 0; r < 3; ++r)
            e[r] = mv(r, 0) * c[0] + mv(r, 1) * c[1] + mv(r, 2) * c[2] + mv(r, 3);
        dist[n] = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    }
    std::vector<size_t> idx(bricks.size());
    std::iota(idx.begin(), idx.end(), size_t(0));
    std::stable_sort(idx.begin(), idx.end(),
                     [&](size_t a, size_t b) { return dist[a] < dist[b]; });
    NodeIds out;
    out.reserve(bricks.size());
    for (size_t i : idx)
        out.push_back(bricks[i]);
    return out;
}

class CudaRayCastRenderer : public Renderer, public DeviceFrameRenderer
{
public:
    /* d_rgba: width * height float RGBA device target (row 0 at the bottom);
     * d_rgba8: optional width * height RGBA8 device buffer for _onFrameEnd;
     * stream: the CUDA stream the frame is ordered on (null: legacy). */
    CudaRayCastRenderer(lv_ctx* ctx, lv_volume* volume, lv_tf* tf, float* d_rgba,
                        uint8_t* d_rgba8 = nullptr, void* stream = nullptr)
        : _ctx(ctx)
        , _volume(volume)
        , _tf(tf)
        , _rgba(d_rgba)
        , _rgba8(d_rgba8)
        , _stream(stream)
    {
        check(lv_volume_get_info(volume, &_info), ctx, "lv_volume_get_info");
    }

    NodeIds order(const NodeIds& bricks, const Frustum& frustum) const override
    {
        return distanceOrder(bricks, frustum, _info);
    }

    void setRenderDesc(const lv_render_desc& desc) override
    {
        _desc = desc;
        _haveDesc = true;
    }
    const lv_frame_stats& frameStats() const override { return _stats; }
    const lv_volume_info& getVolumeInfo() const { return _info; }

protected:
    void _onFrameStart(const Frustum& frustum, const ClipPlanes& planes,
                       const PixelViewport& view, const NodeIds&) override
    {
        if (_haveDesc)
            return;
        RenderParams p;
        p.frameInfo = FrameInfo(frustum, 0, 0);
        p.clipPlanes = planes;
        p.pixelViewPort = view;
        _desc = makeRenderDesc(p);
    }

    void _onFrameRender(const Frustum&, const ClipPlanes&, const PixelViewport&,
                        const NodeIds&) override
    {
        check(lv_render(_ctx, _volume, _tf, &_desc, _rgba, _stream), _ctx, "lv_render");
        check(lv_last_stats(_ctx, &_stats), _ctx, "lv_last_stats");
    }

    void _onFrameEnd(const Frustum&, const ClipPlanes&, const PixelViewport&,
                     const NodeIds&) override
    {
        if (_rgba8)
            check(lv_frame_to_rgba8(_ctx, _rgba, _desc.width, _desc.height, _rgba8, _stream),
                  _ctx, "lv_frame_to_rgba8");
        _haveDesc = false;
    }

private:
    lv_ctx* _ctx;
    lv_volume* _volume;
    lv_tf* _tf;
    float* _rgba;
    uint8_t* _rgba8;
    void* _stream;
    lv_volume_info _info{};
    lv_render_desc _desc{};
    bool _haveDesc = false;
    lv_frame_stats _stats{};
};
} // namespace gb300
} // namespace livre

#endif
