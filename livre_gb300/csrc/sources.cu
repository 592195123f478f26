/*
 * Built-in data sources opened from a URI, like livre::DataSource(uri) with
 * its plugin factory (livre/data/DataSource.cpp:29-63):
 *
 *  - mem://[#w,h,d,block][?datatype=uint8|uint16|...]  (MemoryDataSource,
 *    livre/data/MemoryDataSource.cpp:38-166): every brick is one constant,
 *    (id[0] ^ id[1] ^ id[2] ^ id[3]) + 16 + 127 sin((timeStep + 1) / 200),
 *    overlap 4, default 4096^3 voxels in 32^3 blocks;
 *  - raw://file.raw#x,y,z[,type] and raw://file.nrrd[?output=type]
 *    (RawDataSource, livre/data/RawDataSource.cpp:67-262): one brick holding
 *    the whole file, overlap 0, optional unsigned down-conversion by shifts.
 *
 * Both feed the pool through the same lv_get_data_fn path as user plugins.
 */
#include <dirent.h>
#include <dlfcn.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <regex>
#include <set>
#include <vector>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

#include "lv_runtime.h"

namespace
{
using namespace lv;

struct Uri
{
    std::string scheme, path, query, fragment;
};

Uri parse_uri(const std::string& s)
{
    Uri u;
    /* no scheme: the whole string is a path (a bare file name) */
    const size_t sep = s.find("://");
    std::string rest = s;
    if (sep != std::string::npos)
    {
        u.scheme = s.substr(0, sep);
        rest = s.substr(sep + 3);
    }
    const size_t hash = rest.find('#');
    if (hash != std::string::npos)
    {
        u.fragment = rest.substr(hash + 1);
        rest = rest.substr(0, hash);
    }
    const size_t q = rest.find('?');
    if (q != std::string::npos)
    {
        u.query = rest.substr(q + 1);
        rest = rest.substr(0, q);
    }
    u.path = rest;
    return u;
}

std::string query_value(const std::string& query, const std::string& key)
{
    std::stringstream ss(query);
    std::string kv;
    while (std::getline(ss, kv, '&'))
    {
        const size_t eq = kv.find('=');
        if (eq != std::string::npos && kv.substr(0, eq) == key)
            return kv.substr(eq + 1);
    }
    return "";
}

std::vector<std::string> split(const std::string& s, char c)
{
    std::vector<std::string> out;
    std::stringstream ss(s);
    std::string part;
    while (std::getline(ss, part, c))
        out.push_back(part);
    return out;
}

/* RawDataSource::Impl::getDataType (RawDataSource.cpp:134-150) plus the
 * MemoryDataSource datatype names. */
int parse_type(const std::string& t)
{
    if (t == "char" || t == "int8")
        return LV_DT_INT8;
    if (t == "unsigned char" || t == "uchar" || t == "uint8")
        return LV_DT_UINT8;
    if (t == "short" || t == "int16")
        return LV_DT_INT16;
    if (t == "unsigned short" || t == "ushort" || t == "uint16")
        return LV_DT_UINT16;
    if (t == "int" || t == "int32")
        return LV_DT_INT32;
    if (t == "unsigned int" || t == "uint" || t == "uint32")
        return LV_DT_UINT32;
    if (t == "float")
        return LV_DT_FLOAT;
    return -1;
}

uint32_t type_bytes(int dt)
{
    switch (dt)
    {
    case LV_DT_UINT8:
    case LV_DT_INT8:
        return 1;
    case LV_DT_UINT16:
    case LV_DT_INT16:
        return 2;
    default:
        return 4;
    }
}

/* ---------------------------------------------------------------- mem:// */
struct MemorySource
{
    int dtype;
};

template <class T>
void fill_constant(void* dst, size_t bytes, uint64_t id)
{
    const uint8_t b0 = uint8_t(id), b1 = uint8_t(id >> 8), b2 = uint8_t(id >> 16),
                  b3 = uint8_t(id >> 24);
    const uint32_t t = uint32_t(id >> 46);
    /* computeData (MemoryDataSource.cpp:38-61): int + int + float, converted
     * to the voxel type through a truncating integer conversion */
    const float v = float(int(b0 ^ b1 ^ b2 ^ b3) + 16) +
                    127.0f * std::sin((float(t) + 1.0f) / 200.f);
    T value;
    if (std::is_floating_point<T>::value)
        value = T(v);
    else
        value = T(int64_t(v));
    T* p = static_cast<T*>(dst);
    for (size_t i = 0; i < bytes / sizeof(T); ++i)
        p[i] = value;
}

int memory_get_data(void* user, uint64_t id, void* dst, size_t bytes)
{
    switch (static_cast<MemorySource*>(user)->dtype)
    {
    case LV_DT_UINT8: fill_constant<uint8_t>(dst, bytes, id); break;
    case LV_DT_UINT16: fill_constant<uint16_t>(dst, bytes, id); break;
    case LV_DT_UINT32: fill_constant<uint32_t>(dst, bytes, id); break;
    case LV_DT_INT8: fill_constant<int8_t>(dst, bytes, id); break;
    case LV_DT_INT16: fill_constant<int16_t>(dst, bytes, id); break;
    case LV_DT_INT32: fill_constant<int32_t>(dst, bytes, id); break;
    default: fill_constant<float>(dst, bytes, id); break;
    }
    return 0;
}

void memory_free(void* user) { delete static_cast<MemorySource*>(user); }

/* ---------------------------------------------------------------- raw:// */
struct RawSource
{
    void* map = nullptr;
    size_t map_bytes = 0;
    size_t header = 0;
    int in_type = LV_DT_UINT8, out_type = LV_DT_UINT8;
    size_t voxels = 0;
    ~RawSource()
    {
        if (map)
            munmap(map, map_bytes);
    }
};

template <class I, class O>
void shift_down(const uint8_t* src, void* dst, size_t n)
{
    constexpr int shift = int(sizeof(I) - sizeof(O)) * 8;
    const I* in = reinterpret_cast<const I*>(src);
    O* out = static_cast<O*>(dst);
    for (size_t i = 0; i < n; ++i)
        out[i] = O(in[i] >> shift);
}

int raw_get_data(void* user, uint64_t id, void* dst, size_t bytes)
{
    RawSource* r = static_cast<RawSource*>(user);
    if ((id & 0xFu) != 0)
        return 1; /* single-brick volume: only the root exists */
    const uint8_t* src = static_cast<const uint8_t*>(r->map) + r->header;
    const size_t n = r->voxels;
    if (bytes < n * type_bytes(r->out_type))
        return 1;
    if (r->in_type == r->out_type)
    {
        std::memcpy(dst, src, n * type_bytes(r->in_type));
        return 0;
    }
    /* only unsigned down-conversions (RawDataSource.cpp:108-117) */
    if (r->in_type == LV_DT_UINT16 && r->out_type == LV_DT_UINT8)
        shift_down<uint16_t, uint8_t>(src, dst, n);
    else if (r->in_type == LV_DT_UINT32 && r->out_type == LV_DT_UINT8)
        shift_down<uint32_t, uint8_t>(src, dst, n);
    else if (r->in_type == LV_DT_UINT32 && r->out_type == LV_DT_UINT16)
        shift_down<uint32_t, uint16_t>(src, dst, n);
    else
        return 1;
    return 0;
}

void raw_free(void* user) { delete static_cast<RawSource*>(user); }

bool map_file(RawSource& r, const std::string& file)
{
    const int fd = ::open(file.c_str(), O_RDONLY);
    if (fd < 0)
        return false;
    struct stat st;
    if (fstat(fd, &st) != 0 || st.st_size == 0)
    {
        ::close(fd);
        return false;
    }
    void* p = mmap(nullptr, size_t(st.st_size), PROT_READ, MAP_PRIVATE, fd, 0);
    ::close(fd);
    if (p == MAP_FAILED)
        return false;
    r.map = p;
    r.map_bytes = size_t(st.st_size);
    return true;
}

/* NRRD header: "key: value" lines up to the blank line ending the header. */
bool parse_nrrd(const std::string& file, std::map<std::string, std::string>& kv,
                size_t& header)
{
    std::ifstream in(file, std::ios::binary);
    if (!in)
        return false;
    std::string line;
    if (!std::getline(in, line) || line.compare(0, 4, "NRRD") != 0)
        return false;
    size_t consumed = line.size() + 1;
    while (std::getline(in, line))
    {
        consumed += line.size() + 1;
        if (line.empty() || line == "\r")
            break;
        if (line[0] == '#')
            continue;
        const size_t c = line.find(':');
        if (c == std::string::npos)
            continue;
        std::string key = line.substr(0, c), val = line.substr(c + 1);
        while (!val.empty() && (val[0] == ' ' || val[0] == '='))
            val.erase(0, 1);
        while (!val.empty() && (val.back() == '\r' || val.back() == ' '))
            val.pop_back();
        kv[key] = val;
    }
    header = consumed;
    return true;
}

bool ends_with(const std::string& s, const std::string& e)
{
    return s.size() >= e.size() && s.compare(s.size() - e.size(), e.size(), e) == 0;
}
} // namespace

namespace
{
/* RawDataSource::handles (RawDataSource.cpp:241-252): the raw scheme, or no
 * scheme and a .raw / .img / .nrrd file */
bool is_raw_uri(const Uri& uri)
{
    if (uri.scheme == "raw")
        return true;
    return uri.scheme.empty() && (ends_with(uri.path, ".raw") || ends_with(uri.path, ".img") ||
                                  ends_with(uri.path, ".nrrd"));
}

/* Data sources registered at run time (plugins), in registration order. */
struct SourceEntry
{
    lv_source_handles_fn handles;
    lv_source_open_fn open;
    void* user;
    std::string description;
};
std::mutex g_sources_mutex;
std::vector<SourceEntry>& registered_sources()
{
    static std::vector<SourceEntry> v;
    return v;
}

/* The first registered source that handles `uri` (copied under the lock). */
bool find_source(const char* uri, SourceEntry& out)
{
    std::vector<SourceEntry> copy;
    {
        std::lock_guard<std::mutex> lock(g_sources_mutex);
        copy = registered_sources();
    }
    for (const SourceEntry& e : copy)
        if (e.handles && e.handles(e.user, uri))
        {
            out = e;
            return true;
        }
    return false;
}
} // namespace

extern "C" lv_status lv_register_source(lv_source_handles_fn handles, lv_source_open_fn open,
                                        void* user, const char* description)
{
    if (!handles || !open)
        return LV_EINVAL;
    std::lock_guard<std::mutex> lock(g_sources_mutex);
    registered_sources().push_back(
        SourceEntry{handles, open, user, description ? description : ""});
    return LV_OK;
}

extern "C" lv_status lv_source_descriptions(char* out, size_t capacity, size_t* size)
{
    if (!size)
        return LV_EINVAL;
    /* the registered sources, then the built-in ones, one blank line apart */
    std::string text;
    {
        std::lock_guard<std::mutex> lock(g_sources_mutex);
        for (const SourceEntry& e : registered_sources())
            if (!e.description.empty())
                text += e.description + "\n\n";
    }
    text += "Memory volume: mem://[#w,h,d,block][?datatype=T], one constant value per brick, "
            "overlap 4\n\n"
            "Raw volume: raw://file.raw#x,y,z[,T] or raw://file.nrrd[?output=T], the whole "
            "file as one brick";
    *size = text.size() + 1;
    if (!out)
        return LV_OK; /* size query */
    if (capacity < text.size() + 1)
        return LV_ENOMEM;
    std::memcpy(out, text.c_str(), text.size() + 1);
    return LV_OK;
}

extern "C" lv_status lv_unregister_source(lv_source_handles_fn handles, lv_source_open_fn open)
{
    std::lock_guard<std::mutex> lock(g_sources_mutex);
    auto& v = registered_sources();
    const size_t before = v.size();
    v.erase(std::remove_if(v.begin(), v.end(),
                           [&](const SourceEntry& e) {
                               return e.handles == handles && e.open == open;
                           }),
            v.end());
    return v.size() < before ? LV_OK : LV_ENOTFOUND;
}

extern "C" int lv_source_handles(const char* uri_c)
{
    if (!uri_c)
        return 0;
    SourceEntry e;
    if (find_source(uri_c, e))
        return 1;
    /* MemoryDataSource::handles and RawDataSource::handles
     * (MemoryDataSource.cpp:153-156, RawDataSource.cpp:241-252) */
    const Uri uri = parse_uri(uri_c);
    return uri.scheme == "mem" || is_raw_uri(uri) ? 1 : 0;
}

extern "C" lv_status lv_load_plugins(const char* paths, const char* pattern, uint32_t* n_loaded)
{
    if (n_loaded)
        *n_loaded = 0;
    const char* env = std::getenv("LD_LIBRARY_PATH");
    const std::string dirs = paths ? paths : (env ? env : "");
    std::regex re;
    try
    {
        re = std::regex(pattern ? pattern : "Livre.*Source");
    }
    catch (const std::regex_error&)
    {
        return LV_EINVAL;
    }
    static std::mutex m;
    static std::set<std::string> loaded; /* canonical paths, never unloaded */
    std::lock_guard<std::mutex> lock(m);
    uint32_t count = 0;
    for (const std::string& dir : split(dirs, ':'))
    {
        if (dir.empty())
            continue;
        DIR* d = opendir(dir.c_str());
        if (!d)
            continue;
        std::vector<std::string> names;
        while (const dirent* e = readdir(d))
        {
            const std::string name = e->d_name;
            if (ends_with(name, ".so") && std::regex_search(name, re))
                names.push_back(name);
        }
        closedir(d);
        std::sort(names.begin(), names.end());
        for (const std::string& name : names)
        {
            const std::string path = dir + "/" + name;
            char* real = realpath(path.c_str(), nullptr);
            const std::string key = real ? real : path;
            std::free(real);
            if (loaded.count(key))
                continue;
            if (dlopen(key.c_str(), RTLD_NOW | RTLD_LOCAL))
            {
                loaded.insert(key);
                ++count;
            }
        }
    }
    if (n_loaded)
        *n_loaded = count;
    return LV_OK;
}

namespace
{
/* The data source for `uri`: the first registered source that handles it,
 * else a built-in one. On failure `err` says why and nothing is left open. */
lv_status open_source(const char* uri_c, lv_volume_info& info, lv_get_data_fn& fn, void*& user,
                      void (*&user_free)(void*), std::string& err)
{
    const Uri uri = parse_uri(uri_c);
    info = lv_volume_info{};
    info.comp_count = 1;
    fn = nullptr;
    user = nullptr;
    user_free = nullptr;
    const auto bad = [&err](lv_status st, const std::string& why) {
        err = why;
        return st;
    };
    SourceEntry plugin;
    if (find_source(uri_c, plugin))
    {
        const lv_status st = plugin.open(plugin.user, uri_c, &info, &fn, &user, &user_free);
        if (st != LV_OK)
            return bad(st, std::string("the registered source failed to open ") + uri_c);
    }
    else if (uri.scheme == "mem")
    {
        /* MemoryDataSource::MemoryDataSource (MemoryDataSource.cpp:63-117) */
        int dt = LV_DT_UINT8;
        const std::string t = query_value(uri.query, "datatype");
        if (!t.empty())
            dt = parse_type(t);
        if (dt < 0)
            return bad(LV_EINVAL, "unsupported mem:// datatype " + t);
        if (!query_value(uri.query, "sparsity").empty() &&
            std::atof(query_value(uri.query, "sparsity").c_str()) < 1.0)
            return bad(LV_EINVAL, "mem:// sparsity < 1 is not supported");
        uint32_t dims[3] = {4096, 4096, 4096}, block = 32;
        const std::vector<std::string> p = split(uri.fragment, ',');
        if (p.size() >= 4)
        {
            for (int i = 0; i < 3; ++i)
                dims[i] = uint32_t(std::strtoul(p[i].c_str(), nullptr, 10));
            block = uint32_t(std::strtoul(p[3].c_str(), nullptr, 10));
        }
        if (!dims[0] || !dims[1] || !dims[2] || !block)
            return bad(LV_EINVAL, "invalid mem:// fragment");
        for (int i = 0; i < 3; ++i)
        {
            info.voxels[i] = dims[i];
            info.overlap[i] = 4;
            info.max_block[i] = block + 8;
        }
        info.dtype = uint32_t(dt);
        if (lv_fill_regular_volume_info(&info) != LV_OK)
            return bad(LV_EINVAL, "cannot set up the regular tree");
        MemorySource* m = new MemorySource{dt};
        fn = memory_get_data;
        user = m;
        user_free = memory_free;
    }
    else if (is_raw_uri(uri))
    {
        /* RawDataSource::Impl (RawDataSource.cpp:67-262) */
        RawSource* r = new RawSource();
        const bool is_raw = ends_with(uri.path, ".raw") || ends_with(uri.path, ".img");
        const bool is_nrrd = ends_with(uri.path, ".nrrd");
        int in_type = LV_DT_UINT8;
        uint32_t dims[3] = {0, 0, 0};
        if (is_raw)
        {
            const std::vector<std::string> p = split(uri.fragment, ',');
            if (p.size() < 3)
            {
                delete r;
                return bad(LV_EINVAL, "not enough parameters for the raw file");
            }
            for (int i = 0; i < 3; ++i)
                dims[i] = uint32_t(std::strtoul(p[i].c_str(), nullptr, 10));
            if (p.size() > 3)
                in_type = parse_type(p[3]);
            if (!map_file(*r, uri.path))
            {
                delete r;
                return bad(LV_ENOTFOUND, "cannot mmap file " + uri.path);
            }
        }
        else if (is_nrrd)
        {
            std::map<std::string, std::string> kv;
            size_t header = 0;
            if (!parse_nrrd(uri.path, kv, header))
            {
                delete r;
                return bad(LV_EINVAL, "cannot parse nrrd file " + uri.path);
            }
            std::string data_file = uri.path;
            if (kv.count("data file") || kv.count("datafile"))
            {
                const std::string rel = kv.count("data file") ? kv["data file"] : kv["datafile"];
                const size_t slash = uri.path.find_last_of('/');
                if (!rel.empty() && rel[0] == '/')
                    data_file = rel;
                else
                    data_file = (slash == std::string::npos ? std::string()
                                                            : uri.path.substr(0, slash + 1)) +
                                rel;
                header = 0;
            }
            if (kv.count("encoding") && kv["encoding"] != "raw")
            {
                delete r;
                return bad(LV_EINVAL, "only raw nrrd encoding is supported");
            }
            const std::vector<std::string> sz = split(kv["sizes"], ' ');
            if (sz.size() < 3)
            {
                delete r;
                return bad(LV_EINVAL, "nrrd sizes must have 3 entries");
            }
            for (int i = 0; i < 3; ++i)
                dims[i] = uint32_t(std::strtoul(sz[i].c_str(), nullptr, 10));
            in_type = parse_type(kv["type"]);
            if (!map_file(*r, data_file))
            {
                delete r;
                return bad(LV_ENOTFOUND, "cannot mmap file " + data_file);
            }
            r->header = header;
        }
        else
        {
            delete r;
            return bad(LV_EINVAL, "volume extension does not include raw or nrrd");
        }
        if (in_type < 0 || !dims[0] || !dims[1] || !dims[2])
        {
            delete r;
            return bad(LV_EINVAL, "unsupported raw volume description");
        }
        int out_type = in_type;
        const std::string o = query_value(uri.query, "output");
        if (!o.empty())
            out_type = parse_type(o);
        if (out_type < 0)
        {
            delete r;
            return bad(LV_EINVAL, "unsupported output type " + o);
        }
        r->in_type = in_type;
        r->out_type = out_type;
        r->voxels = size_t(dims[0]) * dims[1] * dims[2];
        if (r->header + r->voxels * type_bytes(in_type) > r->map_bytes)
        {
            delete r;
            return bad(LV_EINVAL, "raw file smaller than its volume");
        }
        const uint32_t maxv = std::max(dims[0], std::max(dims[1], dims[2]));
        info.world_space_per_voxel = 1.0f / float(maxv);
        for (int i = 0; i < 3; ++i)
        {
            info.voxels[i] = dims[i];
            info.max_block[i] = dims[i];
            info.overlap[i] = 0;
            info.world_size[i] = float(dims[i]) * info.world_space_per_voxel;
            info.root_blocks[i] = 1;
        }
        info.depth = 1;
        info.dtype = uint32_t(out_type);
        fn = raw_get_data;
        user = r;
        user_free = raw_free;
    }
    else
        return bad(LV_EINVAL, "no data source handles '" + uri.scheme + "://'");
    return LV_OK;
}
} // namespace

extern "C" lv_status lv_source_open(const char* uri, lv_volume_info* info, lv_get_data_fn* get_data,
                                    void** source, void (**source_free)(void*))
{
    if (!uri || !info || !get_data || !source || !source_free)
        return LV_EINVAL;
    std::string err;
    return open_source(uri, *info, *get_data, *source, *source_free, err);
}

extern "C" lv_status lv_source_probe(const char* uri, lv_volume_info* info)
{
    if (!uri || !info)
        return LV_EINVAL;
    lv_get_data_fn fn = nullptr;
    void* source = nullptr;
    void (*source_free)(void*) = nullptr;
    const lv_status st = lv_source_open(uri, info, &fn, &source, &source_free);
    if (st == LV_OK && source_free)
        source_free(source);
    return st;
}

extern "C" lv_status lv_volume_open(lv_ctx* ctx, const char* uri_c, lv_volume** out)
{
    if (!ctx || !uri_c || !out)
        return fail(ctx, LV_EINVAL, "null argument");
    lv_volume_info info{};
    lv_get_data_fn fn = nullptr;
    void* user = nullptr;
    void (*user_free)(void*) = nullptr;
    std::string err;
    const lv_status opened = open_source(uri_c, info, fn, user, user_free, err);
    if (opened != LV_OK)
        return fail(ctx, opened, err);
    lv_volume* v = nullptr;
    lv_status st = lv_volume_create(ctx, &info, fn, user, &v);
    if (st != LV_OK)
    {
        if (user_free)
            user_free(user);
        return st;
    }
    v->user_free = user_free;
    *out = v;
    return LV_OK;
}

extern "C" lv_status lv_volume_get_data(lv_volume* v, uint64_t node_id, void* dst, size_t bytes)
{
    /* DataSource::getData (livre/data/DataSource.cpp:101-111): invalid ids
     * and nodes outside the octree give no data */
    if (!v || !dst)
        return LV_EINVAL;
    const uint32_t L = nid_level(node_id);
    if (node_id == kInvalidNode || L >= v->info.depth ||
        nid_x(node_id) >= (v->info.root_blocks[0] << L) ||
        nid_y(node_id) >= (v->info.root_blocks[1] << L) ||
        nid_z(node_id) >= (v->info.root_blocks[2] << L))
        return LV_ENOTFOUND;
    if (bytes < v->brick_bytes)
        return LV_EINVAL;
    if (v->kind == SRC_CALLBACK)
        return v->fn(v->user, node_id, dst, v->brick_bytes) == 0 ? LV_OK : LV_ENOTFOUND;
    if (v->kind == SRC_BLOB_HOST)
    {
        const uint64_t idx = node_index(v->level_offset, v->info.root_blocks, node_id);
        std::memcpy(dst, v->host_store.as<uint8_t>() + idx * v->brick_bytes, v->brick_bytes);
        return LV_OK;
    }
    if (v->kind == SRC_FBM_DEVICE) /* the host generator gives the same bytes */
        return lv_fbm_brick(&v->info, &v->fbm, node_id, dst, 0);
    /* device-generated blob bricks */
    lv_ctx* ctx = v->ctx;
    LV_CUDA(ctx, cudaSetDevice(ctx->device));
    DeviceBuffer tmp;
    LV_CUDA(ctx, tmp.reserve(v->brick_bytes));
    lv_status st = lv_blob_generate(ctx, &v->info, &v->blob, &node_id, 1, tmp.ptr, nullptr);
    if (st != LV_OK)
        return st;
    LV_CUDA(ctx, cudaMemcpy(dst, tmp.ptr, v->brick_bytes, cudaMemcpyDeviceToHost));
    return LV_OK;
}
