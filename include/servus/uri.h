/*
 * servus::URI, the subset data-source plugins use to read their URI
 * (scheme://host/path?key=value&...#fragment). Header only.
 */
#ifndef LIVRE_GB300_COMPAT_SERVUS_URI_H
#define LIVRE_GB300_COMPAT_SERVUS_URI_H

#include <map>
#include <string>

namespace servus
{
class URI
{
public:
    URI() = default;
    explicit URI(const std::string& uri) : _text(uri)
    {
        std::string rest = uri;
        const size_t hash = rest.find('#');
        if (hash != std::string::npos)
        {
            _fragment = rest.substr(hash + 1);
            rest = rest.substr(0, hash);
        }
        const size_t q = rest.find('?');
        if (q != std::string::npos)
        {
            _query = rest.substr(q + 1);
            rest = rest.substr(0, q);
            size_t pos = 0;
            while (pos <= _query.size())
            {
                size_t amp = _query.find('&', pos);
                if (amp == std::string::npos)
                    amp = _query.size();
                const std::string kv = _query.substr(pos, amp - pos);
                const size_t eq = kv.find('=');
                if (!kv.empty())
                    _params[kv.substr(0, eq)] = eq == std::string::npos ? "" : kv.substr(eq + 1);
                pos = amp + 1;
            }
        }
        const size_t colon = rest.find("://");
        if (colon != std::string::npos)
        {
            _scheme = rest.substr(0, colon);
            rest = rest.substr(colon + 3);
            const size_t slash = rest.find('/');
            _host = rest.substr(0, slash);
            _path = slash == std::string::npos ? "" : rest.substr(slash);
        }
        else
            _path = rest;
    }
    explicit URI(const char* uri) : URI(std::string(uri)) {}

    const std::string& getScheme() const { return _scheme; }
    const std::string& getHost() const { return _host; }
    const std::string& getPath() const { return _path; }
    const std::string& getQuery() const { return _query; }
    const std::string& getFragment() const { return _fragment; }
    typedef std::map<std::string, std::string>::const_iterator ConstKVIter;
    ConstKVIter queryBegin() const { return _params.begin(); }
    ConstKVIter queryEnd() const { return _params.end(); }
    ConstKVIter findQuery(const std::string& key) const { return _params.find(key); }
    const std::string& str() const { return _text; }

private:
    std::string _text, _scheme, _host, _path, _query, _fragment;
    std::map<std::string, std::string> _params;
};
} // namespace servus

#endif
