/*
 * CPU checks of the renderer interface headers (no device calls): the stage
 * hooks Renderer::render runs for each renderStages value
 * (livre/core/render/Renderer.cpp:33-47), the frustum limits read off a
 * perspective matrix, the matrix inverse, the brick distance order of
 * CudaRayCastRenderer (RayCastRenderer.cpp:57-81) and the render description
 * the pipeline derives from RenderParams (with the coarsest-LOD clamp of
 * RenderPipeline.cpp:71-74 when not idle).
 * Prints "ok" and exits 0 when every check holds.
 */
#include <livre/gb300/CudaRayCastRenderer.h>
#include <livre/lib/pipeline/RenderPipeline.h>

#include <cmath>
#include <cstdio>
#include <string>

namespace
{
int failures = 0;
void expect(bool ok, const char* what)
{
    if (!ok)
    {
        std::printf("FAILED: %s\n", what);
        ++failures;
    }
}

class StageLog : public livre::Renderer
{
public:
    std::string log;
    livre::NodeIds order(const livre::NodeIds& bricks, const livre::Frustum&) const override
    {
        livre::NodeIds r(bricks.rbegin(), bricks.rend());
        return r;
    }

protected:
    void _onFrameStart(const livre::Frustum&, const livre::ClipPlanes&,
                       const livre::PixelViewport&, const livre::NodeIds& b) override
    {
        log += "S" + std::to_string(b.size());
    }
    void _onFrameRender(const livre::Frustum&, const livre::ClipPlanes&,
                        const livre::PixelViewport&, const livre::NodeIds& b) override
    {
        log += "R" + std::to_string(b.empty() ? 0 : b.front().getLevel());
    }
    void _onFrameEnd(const livre::Frustum&, const livre::ClipPlanes&,
                     const livre::PixelViewport&, const livre::NodeIds&) override
    {
        log += "E";
    }
};

livre::Matrix4f perspective(float fovy, float aspect, float n, float f)
{
    livre::Matrix4f p;
    const float t = 1.0f / std::tan(fovy * 0.5f * 3.14159265f / 180.0f);
    p(0, 0) = t / aspect;
    p(1, 1) = t;
    p(2, 2) = (f + n) / (n - f);
    p(2, 3) = 2.0f * f * n / (n - f);
    p(3, 2) = -1.0f;
    p(3, 3) = 0.0f;
    return p;
}
} // namespace

int main()
{
    using namespace livre;
    Matrix4f mv;
    mv(2, 3) = -2.5f; /* translate(0, 0, -2.5) */
    const Matrix4f proj = perspective(45.0f, 1.5f, 0.1f, 15.0f);
    const Frustum fr(mv, proj);
    expect(std::fabs(fr.nearPlane() - 0.1f) < 1e-5f, "near plane");
    expect(std::fabs(fr.farPlane() - 15.0f) < 1e-2f, "far plane");
    const float top = 0.1f * std::tan(22.5f * 3.14159265f / 180.0f);
    expect(std::fabs(fr.top() - top) < 1e-6f && std::fabs(fr.bottom() + top) < 1e-6f,
           "top / bottom");
    expect(std::fabs(fr.right() - 1.5f * top) < 1e-6f, "right");
    expect(std::fabs(fr.getEyePos()[2] - 2.5f) < 1e-6f, "eye position");
    const Matrix4f id = mv * fr.getInvMVMatrix();
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c)
            expect(std::fabs(id(r, c) - (r == c ? 1.0f : 0.0f)) < 1e-6f, "inverse");
    expect(fr.isInFrustum(Boxf(Vector3f(-0.5f), Vector3f(0.5f))), "box in frustum");
    expect(!fr.isInFrustum(Boxf(Vector3f(20.0f), Vector3f(21.0f))), "box outside");

    StageLog r;
    const NodeIds bricks = {NodeId(1, Vector3ui(0, 0, 0)), NodeId(2, Vector3ui(1, 1, 1))};
    const ClipPlanes planes;
    const PixelViewport vp(0, 0, 64, 48);
    r.render(fr, planes, vp, bricks);
    expect(r.log == "S2R2E", "RENDER_ALL: start, render (ordered), end");
    r.log.clear();
    /* a two-pass frame (RenderPipeline.cpp:128-138) */
    r.render(fr, planes, vp, bricks, RENDER_BEGIN | RENDER_FRAME);
    r.render(fr, planes, vp, {bricks[0]}, RENDER_FRAME | RENDER_END);
    expect(r.log == "S2R2R1E", "two passes");
    r.log.clear();
    r.render(fr, planes, vp, bricks, RENDER_FRAME);
    expect(r.log == "R2", "RENDER_FRAME only");

    /* brick distance order: 256^3 in 32^3 bricks + 1 overlap */
    lv_volume_info info{};
    for (int a = 0; a < 3; ++a)
    {
        info.voxels[a] = 256;
        info.max_block[a] = 34;
        info.overlap[a] = 1;
    }
    info.dtype = LV_DT_UINT8;
    info.comp_count = 1;
    expect(lv_fill_regular_volume_info(&info) == LV_OK && info.depth == 4, "volume info");
    NodeIds all;
    for (uint32_t z = 0; z < 2; ++z)
        for (uint32_t y = 0; y < 2; ++y)
            for (uint32_t x = 0; x < 2; ++x)
                all.push_back(NodeId(1, Vector3ui(x, y, z)));
    const NodeIds ord = gb300::distanceOrder(all, fr, info);
    expect(ord.size() == 8, "order keeps every brick");
    expect(ord.front().getPosition()[2] == 1 && ord.back().getPosition()[2] == 0,
           "nearest (z = +) first, farthest last");
    float prev = -1.0f;
    for (const NodeId& n : ord)
    {
        const Vector3f c = gb300::nodeWorldBox(info, n).getCenter();
        const float d = std::sqrt(c[0] * c[0] + c[1] * c[1] + (c[2] - 2.5f) * (c[2] - 2.5f));
        expect(d >= prev - 1e-6f, "distances ascending");
        prev = d;
    }

    RenderParams p;
    p.frameInfo = FrameInfo(fr, 3, 9);
    p.pixelViewPort = PixelViewport(0, 0, 640, 480);
    p.vrParams.setMinLod(1);
    p.vrParams.setMaxLod(5);
    p.vrParams.setSynchronousMode(true);
    p.vrParams.setLinearFiltering(true);
    p.clipPlanes.setPlanes({ClipPlane(0.0f, 1.0f, 0.0f, 0.25f)});
    lv_render_desc d = gb300::makeRenderDesc(p);
    expect(d.width == 640 && d.height == 480 && d.lod.window_height == 480, "viewport");
    expect(d.lod.min_lod == 1 && d.lod.max_lod == 5, "LOD limits when idle");
    expect(d.lod.time_step == 3 && d.synchronous == 1 && d.filter == LV_FILTER_TRILINEAR,
           "time step, residency mode, filter");
    expect(d.lod.n_clip_planes == 1 && d.lod.clip_planes[0][1] == 1.0f &&
               d.lod.clip_planes[0][3] == 0.25f,
           "clip planes");
    expect(d.camera.modelview[14] == -2.5f && d.lod.screen_space_error == 4.0f,
           "camera, default screen-space error");
    p.idle = false;
    d = gb300::makeRenderDesc(p);
    expect(d.lod.max_lod == 1, "interaction: max LOD = min LOD");

    if (failures)
        return 1;
    std::printf("ok\n");
    return 0;
}
