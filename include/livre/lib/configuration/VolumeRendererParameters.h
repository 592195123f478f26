/*
 * livre::VolumeRendererParameters: the renderer settings of
 * livre/lib/zeroeq/volumeRendererParameters.fbs:3-13 in the reference, with
 * the accessor names of its generated class and the same defaults. Header
 * only.
 */
#ifndef LIVRE_GB300_COMPAT_VOLUMERENDERERPARAMETERS_H
#define LIVRE_GB300_COMPAT_VOLUMERENDERERPARAMETERS_H

#include <cstdint>

namespace livre
{
class VolumeRendererParameters
{
public:
    uint32_t getMaxLod() const { return _maxLod; }
    void setMaxLod(uint32_t v) { _maxLod = v; }
    uint32_t getMinLod() const { return _minLod; }
    void setMinLod(uint32_t v) { _minLod = v; }
    float getScreenSpaceError() const { return _sse; }
    void setScreenSpaceError(float v) { _sse = v; }
    bool getSynchronousMode() const { return _synchronous; }
    void setSynchronousMode(bool v) { _synchronous = v; }
    uint32_t getSamplesPerRay() const { return _samplesPerRay; }
    void setSamplesPerRay(uint32_t v) { _samplesPerRay = v; }
    uint64_t getMaxGpuCacheMemory() const { return _maxGpuMB; }
    void setMaxGpuCacheMemory(uint64_t v) { _maxGpuMB = v; }
    uint64_t getMaxCpuCacheMemory() const { return _maxCpuMB; }
    void setMaxCpuCacheMemory(uint64_t v) { _maxCpuMB = v; }
    bool getShowAxes() const { return _showAxes; }
    void setShowAxes(bool v) { _showAxes = v; }
    bool getLinearFiltering() const { return _linear; }
    void setLinearFiltering(bool v) { _linear = v; }

private:
    uint32_t _maxLod = 9; /* (NODEID_LEVEL_BITS << 1) + 1 */
    uint32_t _minLod = 0;
    float _sse = 4.0f;
    bool _synchronous = false;
    uint32_t _samplesPerRay = 0;
    uint64_t _maxGpuMB = 3072;
    uint64_t _maxCpuMB = 8192;
    bool _showAxes = false;
    bool _linear = false;
};
} // namespace livre

#endif
