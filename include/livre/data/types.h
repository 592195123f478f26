/*
 * Value types of Livre's data-source plugin interface, source-compatible
 * with the subset of vmmlib (vmml::vector, vmml::AABB) and of livre/data
 * types that plugins use (livre/data/types.h in the reference). Header only.
 */
#ifndef LIVRE_GB300_COMPAT_TYPES_H
#define LIVRE_GB300_COMPAT_TYPES_H

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

namespace livre
{
/* A 3-component vector with the vmml::vector operations plugins use. */
template <typename T>
class Vector3
{
public:
    Vector3() : _v{T(0), T(0), T(0)} {}
    explicit Vector3(T s) : _v{s, s, s} {}
    Vector3(T x, T y, T z) : _v{x, y, z} {}
    template <typename U>
    Vector3(const Vector3<U>& o) : _v{T(o[0]), T(o[1]), T(o[2])}
    {
    }

    T& operator[](size_t i) { return _v[i]; }
    const T& operator[](size_t i) const { return _v[i]; }
    T x() const { return _v[0]; }
    T y() const { return _v[1]; }
    T z() const { return _v[2]; }
    T find_max() const { return std::max(_v[0], std::max(_v[1], _v[2])); }
    T find_min() const { return std::min(_v[0], std::min(_v[1], _v[2])); }
    /* first index of the largest component */
    size_t find_max_index() const
    {
        size_t m = 0;
        for (size_t i = 1; i < 3; ++i)
            if (_v[i] > _v[m])
                m = i;
        return m;
    }
    T product() const { return _v[0] * _v[1] * _v[2]; }

    Vector3 operator+(const Vector3& o) const { return {_v[0] + o[0], _v[1] + o[1], _v[2] + o[2]}; }
    Vector3 operator-(const Vector3& o) const { return {_v[0] - o[0], _v[1] - o[1], _v[2] - o[2]}; }
    Vector3 operator*(const Vector3& o) const { return {_v[0] * o[0], _v[1] * o[1], _v[2] * o[2]}; }
    Vector3 operator/(const Vector3& o) const { return {_v[0] / o[0], _v[1] / o[1], _v[2] / o[2]}; }
    Vector3 operator+(T s) const { return {_v[0] + s, _v[1] + s, _v[2] + s}; }
    Vector3 operator-(T s) const { return {_v[0] - s, _v[1] - s, _v[2] - s}; }
    Vector3 operator*(T s) const { return {_v[0] * s, _v[1] * s, _v[2] * s}; }
    Vector3 operator/(T s) const { return {_v[0] / s, _v[1] / s, _v[2] / s}; }
    bool operator==(const Vector3& o) const
    {
        return _v[0] == o[0] && _v[1] == o[1] && _v[2] == o[2];
    }
    bool operator!=(const Vector3& o) const { return !(*this == o); }

private:
    T _v[3];
};

typedef Vector3<uint32_t> Vector3ui;
typedef Vector3<int32_t> Vector3i;
typedef Vector3<float> Vector3f;

/* Axis-aligned box [min, max) (vmml::AABB). */
template <typename T>
class Box
{
public:
    Box() = default;
    Box(const Vector3<T>& mn, const Vector3<T>& mx) : _min(mn), _max(mx) {}
    const Vector3<T>& getMin() const { return _min; }
    const Vector3<T>& getMax() const { return _max; }
    Vector3<T> getSize() const { return _max - _min; }
    Vector3<T> getCenter() const { return (_min + _max) * T(0.5); }

private:
    Vector3<T> _min, _max;
};

typedef Box<float> Boxf;
typedef Box<uint32_t> Boxui;
typedef Box<int32_t> Boxi;

/* Voxel data type in a volume (the reference's order, = lv_dtype). */
enum DataType
{
    DT_FLOAT,
    DT_UINT8,
    DT_UINT16,
    DT_UINT32,
    DT_INT8,
    DT_INT16,
    DT_INT32,
    DT_UNDEFINED
};

enum AccessMode
{
    MODE_READ,
    MODE_WRITE,
    MODE_READWRITE
};

class MemoryUnit;
typedef std::shared_ptr<MemoryUnit> MemoryUnitPtr;
typedef std::shared_ptr<const MemoryUnit> ConstMemoryUnitPtr;
} // namespace livre

#endif
