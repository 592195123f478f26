/*
 * A data-source plugin whose getData fails or is slow for some bricks,
 * written against Livre's plugin interface (livre/data/DataSourcePlugin.h,
 * lunchbox::PluginRegisterer) like the reference's plugins. URI:
 * flaky://#edge,block[,sleep_ms]: an edge^3 uint8 volume in block^3 bricks
 * with overlap 1. getData of a brick at x position 1 throws (the upload
 * filter of the reference catches it and skips the brick,
 * DataUploadFilter.cpp:56-64); a brick at y position 1 sleeps sleep_ms
 * milliseconds first (default 20); every brick is filled with
 * 16 + (7 x + 13 y + 29 z + 3 level) mod 200.
 */
#include <chrono>
#include <cstdlib>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <livre/data/DataSourcePlugin.h>
#include <livre/data/MemoryUnit.h>
#include <lunchbox/pluginRegisterer.h>

namespace
{
class FlakyDataSource : public livre::DataSourcePlugin
{
public:
    explicit FlakyDataSource(const livre::DataSourcePluginData& initData)
    {
        std::vector<uint32_t> v;
        std::stringstream ss(initData.getURI().getFragment());
        std::string item;
        while (std::getline(ss, item, ','))
            v.push_back(uint32_t(std::strtoul(item.c_str(), nullptr, 10)));
        if (v.size() < 2)
            throw std::runtime_error("flaky://#edge,block[,sleep_ms]");
        _sleepMs = v.size() > 2 ? v[2] : 20u;
        _volumeInfo.voxels = livre::Vector3ui(v[0]);
        _volumeInfo.overlap = livre::Vector3ui(1u);
        _volumeInfo.maximumBlockSize = livre::Vector3ui(v[1]) + _volumeInfo.overlap * 2u;
        _volumeInfo.dataType = livre::DT_UINT8;
        _volumeInfo.compCount = 1;
        if (!livre::fillRegularVolumeInfo(_volumeInfo))
            throw std::runtime_error("cannot build the octree");
    }

    static bool handles(const livre::DataSourcePluginData& initData)
    {
        return initData.getURI().getScheme() == "flaky";
    }
    static std::string getDescription() { return "test volume with failing and slow bricks"; }

    livre::MemoryUnitPtr getData(const livre::LODNode& node) final
    {
        const livre::Vector3ui p = node.getAbsolutePosition();
        if (p[0] == 1u)
            throw std::runtime_error("brick unavailable");
        if (p[1] == 1u)
            std::this_thread::sleep_for(std::chrono::milliseconds(_sleepMs));
        const uint32_t value =
            16u + (7u * p[0] + 13u * p[1] + 29u * p[2] + 3u * node.getRefLevel()) % 200u;
        const std::vector<uint8_t> out(getVolumeInfo().maximumBlockSize.product(),
                                       uint8_t(value));
        return std::make_shared<livre::AllocMemoryUnit>(out);
    }

private:
    uint32_t _sleepMs = 20;
};

lunchbox::PluginRegisterer<FlakyDataSource> registerer;
} // namespace
