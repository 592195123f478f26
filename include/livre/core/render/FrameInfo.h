/*
 * FrameInfo and NodeAvailability (livre/core/render/FrameInfo.h in the
 * reference): the frustum, time step and id of a frame, and the count of
 * visible bricks a frame could and could not render. Header only.
 */
#ifndef LIVRE_GB300_COMPAT_FRAMEINFO_H
#define LIVRE_GB300_COMPAT_FRAMEINFO_H

#include <livre/data/Frustum.h>

#include <cstddef>
#include <cstdint>

namespace livre
{
struct FrameInfo
{
    FrameInfo(const Frustum& frustum_, uint32_t timeStep_, uint32_t frameId_)
        : frustum(frustum_)
        , timeStep(timeStep_)
        , frameId(frameId_)
    {
    }
    FrameInfo() : frustum(Matrix4f(), Matrix4f()), timeStep(0), frameId(0) {}

    Frustum frustum;   /* the current frustum */
    uint32_t timeStep; /* the time step the data sources deliver */
    uint32_t frameId;  /* the id of the rendered frame */
};

struct NodeAvailability
{
    NodeAvailability() : nAvailable(0), nNotAvailable(0) {}
    NodeAvailability& operator+=(const NodeAvailability& na)
    {
        nAvailable += na.nAvailable;
        nNotAvailable += na.nNotAvailable;
        return *this;
    }
    size_t nAvailable;
    size_t nNotAvailable;
};
} // namespace livre

#endif
