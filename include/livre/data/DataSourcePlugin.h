/*
 * livre::DataSourcePlugin, the interface of Livre's data sources
 * (livre/data/DataSourcePlugin.h:33-109), with the default
 * internalNodeToLODNode of livre/data/DataSourcePlugin.cpp:40-71. A plugin
 * written against the reference compiles against these headers unchanged
 * and registers with lunchbox::PluginRegisterer (lunchbox/pluginRegisterer.h);
 * lv_volume_open then opens its URIs. initializeGL / finishGL are kept and
 * never called (no GL context). Header only.
 */
#ifndef LIVRE_GB300_COMPAT_DATASOURCEPLUGIN_H
#define LIVRE_GB300_COMPAT_DATASOURCEPLUGIN_H

#include <livre/data/LODNode.h>
#include <livre/data/MemoryUnit.h>
#include <livre/data/VolumeInformation.h>
#include <servus/uri.h>

namespace livre
{
class DataSourcePluginData
{
public:
    explicit DataSourcePluginData(const servus::URI& uri, AccessMode mode = MODE_READ)
        : _uri(uri), _accessMode(mode)
    {
    }
    const servus::URI& getURI() const { return _uri; }
    AccessMode getAccessMode() const { return _accessMode; }

private:
    const servus::URI& _uri;
    const AccessMode _accessMode;
};

class DataSourcePlugin
{
public:
    typedef DataSourcePlugin InterfaceT;
    typedef DataSourcePluginData InitDataT;

    DataSourcePlugin() = default;
    virtual ~DataSourcePlugin() = default;
    DataSourcePlugin(const DataSourcePlugin&) = delete;
    DataSourcePlugin& operator=(const DataSourcePlugin&) = delete;

    const VolumeInformation& getVolumeInfo() const { return _volumeInfo; }
    virtual bool initializeGL() { return true; }
    virtual void finishGL() {}
    virtual MemoryUnitPtr getData(const LODNode& node) = 0;

    /* world box: the node's cell of the level's largest brick count, scaled
     * to the world size and centred at the origin */
    virtual LODNode internalNodeToLODNode(const NodeId& node) const
    {
        const Vector3ui bricks = _volumeInfo.rootNode.getBlockSize(node.getLevel());
        const float denom = float(bricks[bricks.find_max_index()]);
        const Vector3f lo = Vector3f(node.getPosition()) / denom;
        const Vector3f hi = Vector3f(node.getPosition() + Vector3ui(1u)) / denom;
        const Vector3f& ws = _volumeInfo.worldSize;
        return LODNode(node, _volumeInfo.maximumBlockSize - _volumeInfo.overlap * 2u,
                       Boxf(lo * ws - ws * 0.5f, hi * ws - ws * 0.5f));
    }
    virtual bool update() { return false; }
    LODNode getNode(const NodeId& nodeId) const { return internalNodeToLODNode(nodeId); }

protected:
    VolumeInformation _volumeInfo;
};
} // namespace livre

#endif
