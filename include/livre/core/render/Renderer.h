/*
 * livre::Renderer (livre/core/render/Renderer.h:38-109 and Renderer.cpp:33-47
 * in the reference): the base class of renderers. render() orders the bricks
 * with order(), then calls the stage hooks its renderStages flags select:
 * _onFrameStart (RENDER_BEGIN), _onFrameRender (RENDER_FRAME), _onFrameEnd
 * (RENDER_END). A multi-pass frame calls render() once per pass with
 * RENDER_BEGIN on the first pass only and RENDER_END on the last.
 * Header only; livre::gb300::CudaRayCastRenderer is this library's subclass.
 */
#ifndef LIVRE_GB300_COMPAT_RENDERER_H
#define LIVRE_GB300_COMPAT_RENDERER_H

#include <livre/core/types.h>
#include <livre/data/Frustum.h>

#include <cstdint>

namespace livre
{
static const uint32_t RENDER_BEGIN = 1u;
static const uint32_t RENDER_FRAME = 1u << 1;
static const uint32_t RENDER_END = 1u << 2;
static const uint32_t RENDER_ALL = RENDER_BEGIN | RENDER_FRAME | RENDER_END;

class Renderer
{
public:
    /* Renders the bricks of one view (or one pass of it). */
    void render(const Frustum& frustum, const ClipPlanes& planes, const PixelViewport& view,
                const NodeIds& bricks, const uint32_t renderStages = RENDER_ALL)
    {
        const NodeIds ordered = order(bricks, frustum);
        if (renderStages & RENDER_BEGIN)
            _onFrameStart(frustum, planes, view, ordered);
        if (renderStages & RENDER_FRAME)
            _onFrameRender(frustum, planes, view, ordered);
        if (renderStages & RENDER_END)
            _onFrameEnd(frustum, planes, view, ordered);
    }

    /* The bricks in the order they are drawn (front to back). */
    virtual NodeIds order(const NodeIds& bricks, const Frustum& frustum) const = 0;

    virtual ~Renderer() {}

protected:
    virtual void _onFrameStart(const Frustum&, const ClipPlanes&, const PixelViewport&,
                               const NodeIds&)
    {
    }
    virtual void _onFrameRender(const Frustum&, const ClipPlanes&, const PixelViewport&,
                                const NodeIds&)
    {
    }
    virtual void _onFrameEnd(const Frustum&, const ClipPlanes&, const PixelViewport&,
                             const NodeIds&)
    {
    }
};
} // namespace livre

#endif
