/*
 * livre::MemoryUnit and its two kinds, as a data-source plugin returns them
 * from getData (livre/data/MemoryUnit.h:33-167): AllocMemoryUnit owns a
 * copy, ConstMemoryUnit shows memory owned elsewhere (e.g. a mapped file).
 * Header only.
 */
#ifndef LIVRE_GB300_COMPAT_MEMORYUNIT_H
#define LIVRE_GB300_COMPAT_MEMORYUNIT_H

#include <cstring>

#include <livre/data/types.h>

namespace livre
{
class MemoryUnit
{
public:
    virtual ~MemoryUnit() = default;
    template <class T>
    const T* getData() const
    {
        return reinterpret_cast<const T*>(_getData());
    }
    template <class T>
    T* getData()
    {
        return reinterpret_cast<T*>(_getData());
    }
    virtual size_t getAllocSize() const = 0;

protected:
    virtual const uint8_t* _getData() const = 0;
    virtual uint8_t* _getData() = 0;
};

class NoMemoryUnit : public MemoryUnit
{
public:
    size_t getAllocSize() const final { return 0; }

private:
    const uint8_t* _getData() const final { return nullptr; }
    uint8_t* _getData() final { return nullptr; }
};

class ConstMemoryUnit : public MemoryUnit
{
public:
    ConstMemoryUnit(const uint8_t* ptr, size_t size) : _ptr(ptr), _size(size) {}
    size_t getAllocSize() const final { return _size; }

protected:
    const uint8_t* _getData() const final { return _ptr; }
    uint8_t* _getData() final { return nullptr; } /* read-only memory */
    const uint8_t* const _ptr;
    const size_t _size;
};

class AllocMemoryUnit : public MemoryUnit
{
public:
    template <typename T>
    AllocMemoryUnit(const T* source, size_t count)
        : _data(reinterpret_cast<const uint8_t*>(source),
                reinterpret_cast<const uint8_t*>(source) + sizeof(T) * count)
    {
    }
    AllocMemoryUnit(const void* source, size_t bytes)
        : _data(static_cast<const uint8_t*>(source), static_cast<const uint8_t*>(source) + bytes)
    {
    }
    template <typename T>
    explicit AllocMemoryUnit(const std::vector<T>& source)
        : AllocMemoryUnit(source.data(), source.size())
    {
    }
    explicit AllocMemoryUnit(size_t bytes) : _data(bytes) {}
    AllocMemoryUnit(const AllocMemoryUnit&) = delete;
    AllocMemoryUnit& operator=(const AllocMemoryUnit&) = delete;
    size_t getAllocSize() const final { return _data.size(); }

private:
    const uint8_t* _getData() const final { return _data.data(); }
    uint8_t* _getData() final { return _data.data(); }
    std::vector<uint8_t> _data;
};
} // namespace livre

#endif
