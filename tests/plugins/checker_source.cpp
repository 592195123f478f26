/*
 * A data-source plugin written against Livre's plugin interface the way the
 * reference's plugins are (livre/data/DataSourcePlugin.h,
 * livre/data/MemoryUnit.h, lunchbox::PluginRegisterer), compiled by the
 * tests against the source-compatible headers in include/. URI:
 * checker://#w,h,d,block[,type]  (type 8 or 16 bits). Voxel (x, y, z) of the
 * finest level holds 40 + 170 * ((x / 16 + y / 16 + z / 16) & 1) (scaled to
 * 16 bits); coarser levels point-sample it at their voxel centres; overlap 1,
 * clamped at the volume edge.
 */
#include <cstdlib>
#include <sstream>
#include <string>
#include <vector>

#include <livre/data/DataSourcePlugin.h>
#include <livre/data/MemoryUnit.h>
#include <lunchbox/pluginRegisterer.h>

namespace
{
class CheckerDataSource : public livre::DataSourcePlugin
{
public:
    explicit CheckerDataSource(const livre::DataSourcePluginData& initData)
    {
        std::vector<uint32_t> v;
        std::stringstream ss(initData.getURI().getFragment());
        std::string item;
        while (std::getline(ss, item, ','))
            v.push_back(uint32_t(std::strtoul(item.c_str(), nullptr, 10)));
        if (v.size() < 4)
            throw std::runtime_error("checker://#w,h,d,block[,bits]");
        _volumeInfo.voxels = livre::Vector3ui(v[0], v[1], v[2]);
        _volumeInfo.overlap = livre::Vector3ui(1u);
        _volumeInfo.maximumBlockSize = livre::Vector3ui(v[3]) + _volumeInfo.overlap * 2u;
        _volumeInfo.dataType = v.size() > 4 && v[4] == 16 ? livre::DT_UINT16 : livre::DT_UINT8;
        _volumeInfo.compCount = 1;
        if (!livre::fillRegularVolumeInfo(_volumeInfo))
            throw std::runtime_error("cannot build the octree");
    }

    static bool handles(const livre::DataSourcePluginData& initData)
    {
        return initData.getURI().getScheme() == "checker";
    }
    static std::string getDescription() { return "checkerboard test volume"; }

    livre::MemoryUnitPtr getData(const livre::LODNode& node) final
    {
        const livre::VolumeInformation& vi = getVolumeInfo();
        const uint32_t depth = vi.rootNode.getDepth();
        const uint32_t s = 1u << (depth - 1u - node.getRefLevel());
        const livre::Vector3ui N = vi.maximumBlockSize;
        const livre::Vector3ui lo = node.getVoxelBox().getMin();
        const bool wide = vi.dataType == livre::DT_UINT16;
        std::vector<uint8_t> out(size_t(N.product()) * (wide ? 2 : 1));
        size_t idx = 0;
        for (uint32_t k = 0; k < N[2]; ++k)
            for (uint32_t j = 0; j < N[1]; ++j)
                for (uint32_t i = 0; i < N[0]; ++i, ++idx)
                {
                    const uint32_t off[3] = {i, j, k};
                    uint32_t f[3];
                    for (int a = 0; a < 3; ++a)
                    {
                        const int32_t last = int32_t((vi.voxels[a] + s - 1u) / s) - 1;
                        int32_t g = int32_t(lo[a] + off[a]) - 1;
                        g = g < 0 ? 0 : (g > last ? last : g);
                        f[a] = uint32_t(g) * s + s / 2u; /* finest voxel at the centre */
                    }
                    const uint32_t v = 40u + 170u * (((f[0] / 16u) + (f[1] / 16u) + (f[2] / 16u)) & 1u);
                    if (wide)
                        reinterpret_cast<uint16_t*>(out.data())[idx] = uint16_t(v * 257u);
                    else
                        out[idx] = uint8_t(v);
                }
        return std::make_shared<livre::AllocMemoryUnit>(out);
    }
};

lunchbox::PluginRegisterer<CheckerDataSource> registerer;
} // namespace
