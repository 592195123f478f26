/*
 * The checks of the reference's data-source test (tests/data/dataSource.cpp:
 * 31-64) written against the source-compatible headers, plus the
 * DataSource::getData / handles / getDescriptions contract. Exit status 0
 * when every check holds; each failure is printed. Arguments: URIs of
 * 1024x1024x512 volumes in 32^3 blocks to test (default the mem:// one).
 */
#include <cstdio>
#include <sstream>
#include <string>

#include <livre/data/DataSource.h>
#include <livre/data/LODNode.h>
#include <livre/data/MemoryUnit.h>
#include <livre/data/NodeId.h>
#include <livre/data/VolumeInformation.h>
#include <servus/uri.h>

namespace
{
int failures = 0;

#define CHECK(cond)                                                        \
    do                                                                     \
    {                                                                      \
        if (!(cond))                                                       \
        {                                                                  \
            std::printf("%s:%d: check failed: %s\n", __FILE__, __LINE__, #cond); \
            ++failures;                                                    \
        }                                                                  \
    } while (0)

const uint32_t BLOCK_SIZE = 32;

void testDataSource(const std::string& uriStr)
{
    const servus::URI uri(uriStr);
    CHECK(livre::DataSource::handles(uri));
    livre::DataSource source(uri);
    const livre::VolumeInformation& info = source.getVolumeInfo();

    /* 32 << depth = 512, the shortest dimension of the volume */
    CHECK(info.rootNode.getDepth() == 5);
    CHECK(info.compCount == 1);

    const livre::NodeId parentNodeId(0, livre::Vector3ui(0, 0, 0), 0);
    const livre::NodeId firstChildNodeId = parentNodeId.getChildren().front();
    const livre::LODNode lodNode = source.getNode(firstChildNodeId);
    CHECK(lodNode.isValid());
    CHECK(lodNode.getVoxelBox().getSize() == livre::Vector3ui(BLOCK_SIZE));
    const livre::Vector3ui blockSize = lodNode.getBlockSize() + info.overlap * 2u;
    CHECK(blockSize == info.maximumBlockSize);

    /* a brick of the octree has data of the full brick size; an invalid id
     * and a node outside the octree have none */
    const livre::ConstMemoryUnitPtr unit =
        static_cast<const livre::DataSource&>(source).getData(firstChildNodeId);
    CHECK(unit && unit->getAllocSize() ==
                      size_t(info.maximumBlockSize.product()) * info.getBytesPerVoxel());
    CHECK(!source.getData(livre::NodeId()));
    CHECK(!source.getData(livre::NodeId(0, livre::Vector3ui(9, 0, 0), 0)));
    CHECK(!source.getData(livre::NodeId(7, livre::Vector3ui(0, 0, 0), 0)));
}
} // namespace

int main(int argc, char** argv)
{
    livre::DataSource::loadPlugins();
    std::stringstream mem;
    mem << "mem://#1024,1024,512," << BLOCK_SIZE;
    if (argc < 2)
        testDataSource(mem.str());
    for (int i = 1; i < argc; ++i)
        testDataSource(argv[i]);

    CHECK(!livre::DataSource::handles(servus::URI("nosuchscheme://volume")));
    CHECK(livre::DataSource::handles(servus::URI("volume.nrrd")));
    CHECK(livre::DataSource::getDescriptions().find("mem://") != std::string::npos);
    bool threw = false;
    try
    {
        livre::DataSource bad(servus::URI("nosuchscheme://volume"));
    }
    catch (const std::runtime_error&)
    {
        threw = true;
    }
    CHECK(threw);
    std::printf("%d failure(s)\n", failures);
    return failures == 0 ? 0 : 1;
}
