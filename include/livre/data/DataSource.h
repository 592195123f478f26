/*
 * livre::DataSource (livre/data/DataSource.h:30-110,
 * livre/data/DataSource.cpp:29-111): the data source for a URI, opened
 * through the library's source table (registered plugins in registration
 * order, then mem:// and raw://) and read on the host, without a render
 * context or a device. Nodes map to LODNodes by the default rule of
 * DataSourcePlugin::internalNodeToLODNode. initializeGL / finishGL do
 * nothing (no GL context). Header only (links liblivre_gb300).
 */
#ifndef LIVRE_GB300_COMPAT_DATASOURCE_H
#define LIVRE_GB300_COMPAT_DATASOURCE_H

#include <stdexcept>
#include <string>

#include <livre/data/LODNode.h>
#include <livre/data/MemoryUnit.h>
#include <livre/data/VolumeInformation.h>
#include <servus/uri.h>

namespace livre
{
class DataSource
{
public:
    explicit DataSource(const servus::URI& uri, AccessMode accessMode = MODE_READ)
    {
        if (accessMode != MODE_READ)
            throw std::runtime_error("only read access is supported: " + uri.str());
        lv_volume_info v{};
        if (lv_source_open(uri.str().c_str(), &v, &_getData, &_source, &_free) != LV_OK)
            throw std::runtime_error("no data source opens " + uri.str());
        _info = fromLvInfo(v);
        _brickBytes = size_t(v.max_block[0]) * v.max_block[1] * v.max_block[2] *
                      _info.getBytesPerVoxel() * _info.compCount;
    }
    ~DataSource()
    {
        if (_free)
            _free(_source);
    }
    DataSource(const DataSource&) = delete;
    DataSource& operator=(const DataSource&) = delete;

    /* loads the plugin libraries named Livre*Source on LD_LIBRARY_PATH */
    static void loadPlugins() { lv_load_plugins(nullptr, nullptr, nullptr); }

    static std::string getDescriptions()
    {
        size_t n = 0;
        if (lv_source_descriptions(nullptr, 0, &n) != LV_OK)
            return std::string();
        std::string text(n, '\0');
        if (lv_source_descriptions(&text[0], n, &n) != LV_OK)
            return std::string();
        text.resize(n - 1);
        return text;
    }

    static bool handles(const servus::URI& uri)
    {
        return lv_source_handles(uri.str().c_str()) != 0;
    }

    const VolumeInformation& getVolumeInfo() const { return _info; }

    static VolumeInformation getVolumeInfo(const servus::URI& uri)
    {
        return DataSource(uri).getVolumeInfo();
    }

    bool initializeGL() { return true; }
    void finishGL() {}
    bool update() { return false; }

    /* null for an invalid node, one outside the octree, or one the source
     * has no data for */
    MemoryUnitPtr getData(const NodeId& nodeId)
    {
        if (!inTree(nodeId))
            return MemoryUnitPtr();
        std::shared_ptr<AllocMemoryUnit> unit = std::make_shared<AllocMemoryUnit>(_brickBytes);
        if (_getData(_source, nodeId.getId(), unit->getData<uint8_t>(), _brickBytes) != 0)
            return MemoryUnitPtr();
        return unit;
    }
    ConstMemoryUnitPtr getData(const NodeId& nodeId) const
    {
        return const_cast<DataSource*>(this)->getData(nodeId);
    }

    LODNode getNode(const NodeId& node) const
    {
        if (!node.isValid())
            return LODNode();
        const Vector3ui bricks = _info.rootNode.getBlockSize(node.getLevel());
        const float denom = float(bricks[bricks.find_max_index()]);
        const Vector3f lo = Vector3f(node.getPosition()) / denom;
        const Vector3f hi = Vector3f(node.getPosition() + Vector3ui(1u)) / denom;
        const Vector3f& ws = _info.worldSize;
        return LODNode(node, _info.maximumBlockSize - _info.overlap * 2u,
                       Boxf(lo * ws - ws * 0.5f, hi * ws - ws * 0.5f));
    }

private:
    bool inTree(const NodeId& node) const
    {
        if (!node.isValid() || node.getLevel() >= _info.rootNode.getDepth())
            return false;
        const Vector3ui bricks = _info.rootNode.getBlockSize(node.getLevel());
        const Vector3ui p = node.getPosition();
        return p[0] < bricks[0] && p[1] < bricks[1] && p[2] < bricks[2];
    }

    VolumeInformation _info;
    size_t _brickBytes = 0;
    lv_get_data_fn _getData = nullptr;
    void* _source = nullptr;
    void (*_free)(void*) = nullptr;
};
} // namespace livre

#endif
