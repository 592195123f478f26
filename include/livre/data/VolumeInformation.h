/*
 * livre::VolumeInformation and RootNode (livre/data/VolumeInformation.h,
 * livre/data/NodeId.h:166-199) with the fields plugins fill, and
 * fillRegularVolumeInfo (livre/data/DataSourcePlugin.cpp:73-95), evaluated by
 * the library (lv_fill_regular_volume_info) so the octree matches the one
 * the renderer builds. Header only (links liblivre_gb300).
 */
#ifndef LIVRE_GB300_COMPAT_VOLUMEINFORMATION_H
#define LIVRE_GB300_COMPAT_VOLUMEINFORMATION_H

#include <livre/data/NodeId.h>
#include <livre_gb300.h>

namespace livre
{
class RootNode
{
public:
    RootNode() = default;
    RootNode(uint32_t depth, const Vector3ui& blockSize) : _depth(depth), _blocks(blockSize) {}
    uint32_t getDepth() const { return _depth; }
    const Vector3ui& getBlockSize() const { return _blocks; }
    /* bricks per axis at `level` */
    Vector3ui getBlockSize(uint32_t level) const
    {
        return Vector3ui(_blocks[0] << level, _blocks[1] << level, _blocks[2] << level);
    }

private:
    uint32_t _depth = 0;
    Vector3ui _blocks;
};

struct VolumeInformation
{
    bool bigEndian = false;
    uint32_t compCount = 1;
    DataType dataType = DT_UINT8;
    Vector3ui overlap;
    Vector3ui maximumBlockSize;
    Vector3ui voxels;
    Vector3f worldSize;
    Vector3f resolution{-1.0f, -1.0f, -1.0f};
    float worldSpacePerVoxel = 1.0f;
    float meterToDataUnitRatio = 1.0f;
    RootNode rootNode;

    size_t getBytesPerVoxel() const
    {
        switch (dataType)
        {
        case DT_UINT8:
        case DT_INT8: return 1;
        case DT_UINT16:
        case DT_INT16: return 2;
        default: return 4;
        }
    }
};

/* The library's form of the same description. */
inline lv_volume_info toLvInfo(const VolumeInformation& info)
{
    lv_volume_info v{};
    for (int a = 0; a < 3; ++a)
    {
        v.voxels[a] = info.voxels[a];
        v.max_block[a] = info.maximumBlockSize[a];
        v.overlap[a] = info.overlap[a];
    }
    v.dtype = uint32_t(info.dataType);
    v.comp_count = info.compCount;
    return v;
}

/* A description the library filled (lv_fill_regular_volume_info applied). */
inline VolumeInformation fromLvInfo(const lv_volume_info& v)
{
    VolumeInformation info;
    info.voxels = Vector3ui(v.voxels[0], v.voxels[1], v.voxels[2]);
    info.maximumBlockSize = Vector3ui(v.max_block[0], v.max_block[1], v.max_block[2]);
    info.overlap = Vector3ui(v.overlap[0], v.overlap[1], v.overlap[2]);
    info.dataType = DataType(v.dtype);
    info.compCount = v.comp_count;
    info.worldSpacePerVoxel = v.world_space_per_voxel;
    info.worldSize = Vector3f(v.world_size[0], v.world_size[1], v.world_size[2]);
    info.rootNode =
        RootNode(v.depth, Vector3ui(v.root_blocks[0], v.root_blocks[1], v.root_blocks[2]));
    return info;
}

inline bool fillRegularVolumeInfo(VolumeInformation& info)
{
    lv_volume_info v = toLvInfo(info);
    if (lv_fill_regular_volume_info(&v) != LV_OK)
        return false;
    info.worldSpacePerVoxel = v.world_space_per_voxel;
    info.worldSize = Vector3f(v.world_size[0], v.world_size[1], v.world_size[2]);
    info.rootNode =
        RootNode(v.depth, Vector3ui(v.root_blocks[0], v.root_blocks[1], v.root_blocks[2]));
    return true;
}
} // namespace livre

#endif
