/*
 * Value types of Livre's data-source plugin interface, source-compatible
 * with the subset of vmmlib (vmml::vector, vmml::AABB) and of livre/data
 * types that plugins use (livre/data/types.h in the reference). Header only.
 */
#ifndef LIVRE_GB300_COMPAT_TYPES_H
#define LIVRE_GB300_COMPAT_TYPES_H

#include <algorithm>
#include <array>
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

/* An N-component vector (vmml::vector) for the renderer interface's pixel
 * viewports, viewports and planes. */
template <size_t N, typename T>
class VectorN
{
public:
    VectorN() { std::fill(_v, _v + N, T(0)); }
    explicit VectorN(T s) { std::fill(_v, _v + N, s); }
    VectorN(T x, T y) : _v{x, y} { static_assert(N == 2, "2 components"); }
    VectorN(T x, T y, T z, T w) : _v{x, y, z, w} { static_assert(N == 4, "4 components"); }
    T& operator[](size_t i) { return _v[i]; }
    const T& operator[](size_t i) const { return _v[i]; }
    bool operator==(const VectorN& o) const { return std::equal(_v, _v + N, o._v); }
    bool operator!=(const VectorN& o) const { return !(*this == o); }
    const T* data() const { return _v; }

private:
    T _v[N];
};

typedef VectorN<2, float> Vector2f;
typedef VectorN<2, int32_t> Vector2i;
typedef VectorN<4, float> Vector4f;
typedef VectorN<4, int32_t> Vector4i;
typedef VectorN<4, uint32_t> Vector4ui;

/* x, y, width, height in pixels (vmml::Vector4i as the reference uses it) */
typedef Vector4i PixelViewport;
/* x, y, width, height relative to the destination channel */
typedef Vector4f Viewport;
/* a plane (a, b, c, d): a*x + b*y + c*z + d >= 0 on its inside */
typedef Vector4f Plane;
/* a data range [min, max] in [0, 1] (livre/data/types.h:50) */
typedef std::array<float, 2> Range;

/* A 4x4 float matrix, column major (vmml::Matrix4f: element (row, column)
 * at array[column * 4 + row]). */
class Matrix4f
{
public:
    float array[16];

    Matrix4f() : array{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1} {}
    explicit Matrix4f(const float* columnMajor) { std::copy(columnMajor, columnMajor + 16, array); }

    float& operator()(size_t row, size_t col) { return array[col * 4 + row]; }
    float operator()(size_t row, size_t col) const { return array[col * 4 + row]; }

    Matrix4f operator*(const Matrix4f& o) const
    {
        Matrix4f r;
        for (size_t row = 0; row < 4; ++row)
            for (size_t col = 0; col < 4; ++col)
            {
                float acc = 0.0f;
                for (size_t k = 0; k < 4; ++k)
                    acc += (*this)(row, k) * o(k, col);
                r(row, col) = acc;
            }
        return r;
    }
    bool operator==(const Matrix4f& o) const { return std::equal(array, array + 16, o.array); }
    bool operator!=(const Matrix4f& o) const { return !(*this == o); }

    Vector4f getColumn(size_t c) const
    {
        return Vector4f(array[c * 4], array[c * 4 + 1], array[c * 4 + 2], array[c * 4 + 3]);
    }
    Vector3f getTranslation() const { return Vector3f(array[12], array[13], array[14]); }

    Matrix4f transposed() const
    {
        Matrix4f r;
        for (size_t row = 0; row < 4; ++row)
            for (size_t col = 0; col < 4; ++col)
                r(row, col) = (*this)(col, row);
        return r;
    }

    /* The inverse by cofactors (2x2 minors of the first two and the last two
     * rows); false for a singular matrix. */
    bool inverse(Matrix4f& out) const
    {
        const Matrix4f& m = *this;
        const float s0 = m(0, 0) * m(1, 1) - m(1, 0) * m(0, 1);
        const float s1 = m(0, 0) * m(1, 2) - m(1, 0) * m(0, 2);
        const float s2 = m(0, 0) * m(1, 3) - m(1, 0) * m(0, 3);
        const float s3 = m(0, 1) * m(1, 2) - m(1, 1) * m(0, 2);
        const float s4 = m(0, 1) * m(1, 3) - m(1, 1) * m(0, 3);
        const float s5 = m(0, 2) * m(1, 3) - m(1, 2) * m(0, 3);
        const float c5 = m(2, 2) * m(3, 3) - m(3, 2) * m(2, 3);
        const float c4 = m(2, 1) * m(3, 3) - m(3, 1) * m(2, 3);
        const float c3 = m(2, 1) * m(3, 2) - m(3, 1) * m(2, 2);
        const float c2 = m(2, 0) * m(3, 3) - m(3, 0) * m(2, 3);
        const float c1 = m(2, 0) * m(3, 2) - m(3, 0) * m(2, 2);
        const float c0 = m(2, 0) * m(3, 1) - m(3, 0) * m(2, 1);
        const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
        if (det == 0.0f)
            return false;
        const float k = 1.0f / det;
        out(0, 0) = (m(1, 1) * c5 - m(1, 2) * c4 + m(1, 3) * c3) * k;
        out(0, 1) = (-m(0, 1) * c5 + m(0, 2) * c4 - m(0, 3) * c3) * k;
        out(0, 2) = (m(3, 1) * s5 - m(3, 2) * s4 + m(3, 3) * s3) * k;
        out(0, 3) = (-m(2, 1) * s5 + m(2, 2) * s4 - m(2, 3) * s3) * k;
        out(1, 0) = (-m(1, 0) * c5 + m(1, 2) * c2 - m(1, 3) * c1) * k;
        out(1, 1) = (m(0, 0) * c5 - m(0, 2) * c2 + m(0, 3) * c1) * k;
        out(1, 2) = (-m(3, 0) * s5 + m(3, 2) * s2 - m(3, 3) * s1) * k;
        out(1, 3) = (m(2, 0) * s5 - m(2, 2) * s2 + m(2, 3) * s1) * k;
        out(2, 0) = (m(1, 0) * c4 - m(1, 1) * c2 + m(1, 3) * c0) * k;
        out(2, 1) = (-m(0, 0) * c4 + m(0, 1) * c2 - m(0, 3) * c0) * k;
        out(2, 2) = (m(3, 0) * s4 - m(3, 1) * s2 + m(3, 3) * s0) * k;
        out(2, 3) = (-m(2, 0) * s4 + m(2, 1) * s2 - m(2, 3) * s0) * k;
        out(3, 0) = (-m(1, 0) * c3 + m(1, 1) * c1 - m(1, 2) * c0) * k;
        out(3, 1) = (m(0, 0) * c3 - m(0, 1) * c1 + m(0, 2) * c0) * k;
        out(3, 2) = (-m(3, 0) * s3 + m(3, 1) * s1 - m(3, 2) * s0) * k;
        out(3, 3) = (m(2, 0) * s3 - m(2, 1) * s1 + m(2, 2) * s0) * k;
        return true;
    }
    Matrix4f inverse() const
    {
        Matrix4f r;
        inverse(r);
        return r;
    }
};
} // namespace livre

#endif
