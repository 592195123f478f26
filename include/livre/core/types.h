/*
 * Value types of Livre's renderer interface (livre/core/types.h in the
 * reference) that a Renderer subclass and the render pipeline use: NodeIds,
 * pixel viewports and the clip planes of lexis::render::ClipPlanes (the
 * getPlanes / getNormal / getD accessors RayCastRenderer.cpp:342-366 reads).
 * Header only.
 */
#ifndef LIVRE_GB300_COMPAT_CORE_TYPES_H
#define LIVRE_GB300_COMPAT_CORE_TYPES_H

#include <livre/data/NodeId.h>
#include <livre/data/types.h>

#include <vector>

namespace livre
{
/* One clip plane: points p with normal . p + d >= 0 are kept. */
class ClipPlane
{
public:
    ClipPlane() : _n{0.0f, 0.0f, 0.0f}, _d(0.0f) {}
    ClipPlane(float nx, float ny, float nz, float d) : _n{nx, ny, nz}, _d(d) {}
    const float* getNormal() const { return _n; }
    float getD() const { return _d; }

private:
    float _n[3];
    float _d;
};

/* Up to six clip planes of a view (lexis::render::ClipPlanes). */
class ClipPlanes
{
public:
    ClipPlanes() = default;
    explicit ClipPlanes(const std::vector<ClipPlane>& planes) : _planes(planes) {}
    const std::vector<ClipPlane>& getPlanes() const { return _planes; }
    void setPlanes(const std::vector<ClipPlane>& planes) { _planes = planes; }
    void clear() { _planes.clear(); }

    /* True if the box lies entirely on the discarded side of a plane. */
    bool isOutside(const Boxf& box) const
    {
        for (const ClipPlane& p : _planes)
        {
            float v = p.getD();
            for (size_t i = 0; i < 3; ++i)
                v += p.getNormal()[i] *
                     (p.getNormal()[i] >= 0.0f ? box.getMax()[i] : box.getMin()[i]);
            if (v < 0.0f)
                return true;
        }
        return false;
    }

private:
    std::vector<ClipPlane> _planes;
};
} // namespace livre

#endif
