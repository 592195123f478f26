/*
 * lunchbox::PluginRegisterer<T>: a static instance in a data-source plugin
 * registers T with the library (the reference's plugin registration,
 * livre/data/DataSource.cpp:29-63), so lv_volume_open opens the URIs that
 * T::handles accepts. getData is called one brick at a time per volume (a
 * plugin need not be thread-safe); a null or short MemoryUnit means the
 * node has no data, as in the reference. Header only.
 */
#ifndef LIVRE_GB300_COMPAT_PLUGINREGISTERER_H
#define LIVRE_GB300_COMPAT_PLUGINREGISTERER_H

#include <cstring>
#include <memory>
#include <mutex>

#include <livre/data/DataSourcePlugin.h>

namespace lunchbox
{
template <class T>
class PluginRegisterer
{
public:
    PluginRegisterer()
    {
        lv_register_source(&handles, &open, nullptr, T::getDescription().c_str());
    }
    ~PluginRegisterer() { lv_unregister_source(&handles, &open); }
    PluginRegisterer(const PluginRegisterer&) = delete;
    PluginRegisterer& operator=(const PluginRegisterer&) = delete;

private:
    struct Source
    {
        explicit Source(const char* text) : uri(text), data(uri), plugin(new T(data)) {}
        servus::URI uri;
        livre::DataSourcePluginData data; /* refers to uri */
        std::unique_ptr<T> plugin;
        std::mutex m;
    };

    static int handles(void*, const char* uri)
    {
        try
        {
            const servus::URI u(uri);
            return T::handles(livre::DataSourcePluginData(u)) ? 1 : 0;
        }
        catch (...)
        {
            return 0;
        }
    }

    static lv_status open(void*, const char* uri, lv_volume_info* info, lv_get_data_fn* get_data,
                          void** source, void (**source_free)(void*))
    {
        Source* s = nullptr;
        try
        {
            s = new Source(uri);
        }
        catch (...)
        {
            return LV_EINVAL;
        }
        *info = livre::toLvInfo(s->plugin->getVolumeInfo());
        if (lv_fill_regular_volume_info(info) != LV_OK)
        {
            delete s;
            return LV_EINVAL;
        }
        *get_data = &getData;
        *source = s;
        *source_free = &destroy;
        return LV_OK;
    }

    static int getData(void* user, uint64_t id, void* dst, size_t bytes)
    {
        Source* s = static_cast<Source*>(user);
        std::lock_guard<std::mutex> lock(s->m);
        try
        {
            const livre::ConstMemoryUnitPtr unit =
                s->plugin->getData(s->plugin->getNode(livre::NodeId(id)));
            if (!unit || unit->getAllocSize() < bytes)
                return 1;
            std::memcpy(dst, unit->getData<uint8_t>(), bytes);
            return 0;
        }
        catch (...)
        {
            return 1;
        }
    }

    static void destroy(void* user) { delete static_cast<Source*>(user); }
};
} // namespace lunchbox

#endif
