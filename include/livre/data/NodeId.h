/*
 * livre::NodeId: a brick of the octree as one 64-bit id (level 4 bits, x / y
 * / z 14 bits each, time step 18 bits; all ones is invalid), the packing and
 * child order of the reference (livre/data/NodeId.h:31-160,
 * livre/data/NodeId.cpp:23-163) so ids pass unchanged between plugins, the
 * C ABI and the device. Header only.
 */
#ifndef LIVRE_GB300_COMPAT_NODEID_H
#define LIVRE_GB300_COMPAT_NODEID_H

#include <livre/data/types.h>

namespace livre
{
class NodeId
{
public:
    static constexpr uint64_t INVALID = ~uint64_t(0);

    NodeId() : _id(INVALID) {}
    explicit NodeId(uint64_t id) : _id(id) {}
    NodeId(uint32_t level, const Vector3ui& pos, uint32_t frame = 0)
        : _id(uint64_t(level & 0xFu) | (uint64_t(pos[0] & 0x3FFFu) << 4) |
              (uint64_t(pos[1] & 0x3FFFu) << 18) | (uint64_t(pos[2] & 0x3FFFu) << 32) |
              (uint64_t(frame & 0x3FFFFu) << 46))
    {
    }

    uint64_t getId() const { return _id; }
    uint32_t getLevel() const { return uint32_t(_id & 0xFu); }
    Vector3ui getPosition() const
    {
        return Vector3ui(uint32_t((_id >> 4) & 0x3FFFu), uint32_t((_id >> 18) & 0x3FFFu),
                         uint32_t((_id >> 32) & 0x3FFFu));
    }
    uint32_t getTimeStep() const { return uint32_t(_id >> 46); }
    uint32_t getFrame() const { return getTimeStep(); }
    bool isValid() const { return getLevel() != 0xFu; } /* INVALID_LEVEL */
    bool isRoot() const { return isValid() && getLevel() == 0; }

    NodeId getParent() const
    {
        if (!isValid() || getLevel() == 0)
            return NodeId();
        const Vector3ui p = getPosition();
        return NodeId(getLevel() - 1, Vector3ui(p[0] / 2, p[1] / 2, p[2] / 2), getTimeStep());
    }
    /* x outer, then y, then z (NodeId.cpp:92-114) */
    std::vector<NodeId> getChildren() const
    {
        std::vector<NodeId> c;
        if (!isValid())
            return c;
        const Vector3ui p = getPosition() * 2u;
        for (uint32_t x = 0; x < 2; ++x)
            for (uint32_t y = 0; y < 2; ++y)
                for (uint32_t z = 0; z < 2; ++z)
                    c.emplace_back(getLevel() + 1, p + Vector3ui(x, y, z), getTimeStep());
        return c;
    }

    bool operator==(const NodeId& o) const { return _id == o._id; }
    bool operator!=(const NodeId& o) const { return _id != o._id; }
    bool operator<(const NodeId& o) const { return _id < o._id; }

private:
    uint64_t _id;
};

typedef std::vector<NodeId> NodeIds;
} // namespace livre

#endif
