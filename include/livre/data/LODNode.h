/*
 * livre::LODNode: a node id with its voxel box and world box
 * (livre/data/LODNode.h, livre/data/LODNode.cpp:30-64). Header only.
 */
#ifndef LIVRE_GB300_COMPAT_LODNODE_H
#define LIVRE_GB300_COMPAT_LODNODE_H

#include <livre/data/NodeId.h>

namespace livre
{
class LODNode
{
public:
    LODNode() : _blockSize(0u) {}
    /* world box in [0, 1] units of the level's largest brick count */
    LODNode(const NodeId& nodeId, const Vector3ui& blockSize,
            const Vector3ui& levelTotalBlockDimensions)
        : _nodeId(nodeId), _blockSize(blockSize), _voxelBox(localBox())
    {
        const Vector3f lo(getAbsolutePosition());
        const Vector3f hi(getAbsolutePosition() + Vector3ui(1u));
        const float denom = float(levelTotalBlockDimensions[levelTotalBlockDimensions.find_max_index()]);
        _worldBox = Boxf(lo / denom, hi / denom);
    }
    LODNode(const NodeId& nodeId, const Vector3ui& blockSize, const Boxf& worldBox)
        : _nodeId(nodeId), _blockSize(blockSize), _voxelBox(localBox()), _worldBox(worldBox)
    {
    }

    Vector3ui getAbsolutePosition() const { return _nodeId.getPosition(); }
    Vector3f getRelativePosition() const
    {
        return Vector3f(getAbsolutePosition()) / float(1u << getRefLevel());
    }
    const Boxui& getVoxelBox() const { return _voxelBox; }
    const Boxf& getWorldBox() const { return _worldBox; }
    uint32_t getRefLevel() const { return _nodeId.getLevel(); }
    NodeId getNodeId() const { return _nodeId; }
    bool isValid() const { return _nodeId.isValid(); }
    const Vector3ui& getBlockSize() const { return _blockSize; }
    bool operator==(const LODNode& o) const { return _nodeId == o._nodeId; }

private:
    Boxui localBox() const
    {
        const Vector3ui p = getAbsolutePosition() * _blockSize;
        return Boxui(p, p + _blockSize);
    }
    NodeId _nodeId;
    Vector3ui _blockSize;
    Boxui _voxelBox;
    Boxf _worldBox;
};
} // namespace livre

#endif
