/*
 * livre::Frustum (livre/data/Frustum.h, Frustum.cpp:24-76 in the reference):
 * the viewing frustum of one view from its modelview and projection
 * matrices, with the accessors the renderer interface uses. Header only.
 *
 * The frustum limits (left, right, bottom, top, near, far) are read off a
 * perspective projection matrix; the culling planes are the Gribb-Hartmann
 * planes of projection * modelview, normalised, tested with the box corner
 * farthest along each normal. The device LOD selection
 * (lv_select_visible, lv_render) does its own culling from the same two
 * matrices; this class does not feed it.
 */
#ifndef LIVRE_GB300_COMPAT_FRUSTUM_H
#define LIVRE_GB300_COMPAT_FRUSTUM_H

#include <livre/data/types.h>

#include <cmath>

namespace livre
{
class Frustum
{
public:
    Frustum(const Matrix4f& modelViewMatrix, const Matrix4f& projectionMatrix)
        : _mv(modelViewMatrix)
        , _proj(projectionMatrix)
    {
        _mv.inverse(_invMV);
        _proj.inverse(_invProj);
        _eye = _invMV.getTranslation();
        const Vector4f d = _invMV.getColumn(2);
        _dir = Vector3f(d[0], d[1], d[2]);
        /* a perspective matrix: P(2,2) = (f + n) / (n - f),
         * P(2,3) = 2 f n / (n - f), P(0,0) = 2n / (r - l), P(0,2) = (r + l) / (r - l) */
        const float a = _proj(2, 2), b = _proj(2, 3);
        _near = b / (a - 1.0f);
        _far = b / (a + 1.0f);
        _left = _near * (_proj(0, 2) - 1.0f) / _proj(0, 0);
        _right = _near * (_proj(0, 2) + 1.0f) / _proj(0, 0);
        _bottom = _near * (_proj(1, 2) - 1.0f) / _proj(1, 1);
        _top = _near * (_proj(1, 2) + 1.0f) / _proj(1, 1);
        const Matrix4f c = _proj * _mv;
        /* left, right, bottom, top, near, far: row 3 +- rows 0, 1, 2 */
        for (int p = 0; p < 6; ++p)
        {
            const int row = p / 2;
            const float sgn = (p % 2) ? -1.0f : 1.0f;
            float q[4];
            for (int k = 0; k < 4; ++k)
                q[k] = c(3, k) + sgn * c(row, k);
            const float len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
            _planes[p] = Plane(q[0] / len, q[1] / len, q[2] / len, q[3] / len);
        }
    }

    const Matrix4f& getMVMatrix() const { return _mv; }
    const Matrix4f& getProjMatrix() const { return _proj; }
    const Matrix4f& getInvMVMatrix() const { return _invMV; }
    const Matrix4f& getInvProjMatrix() const { return _invProj; }
    Matrix4f getMVPMatrix() const { return _proj * _mv; }
    Matrix4f getNormalMatrix() const { return _invMV.transposed(); }
    const Vector3f& getEyePos() const { return _eye; }
    const Vector3f& getViewDir() const { return _dir; }
    const Plane& getNearPlane() const { return _planes[4]; }

    float left() const { return _left; }
    float right() const { return _right; }
    float bottom() const { return _bottom; }
    float top() const { return _top; }
    float nearPlane() const { return _near; }
    float farPlane() const { return _far; }

    /* True if the box is inside or intersects the frustum. */
    bool isInFrustum(const Boxf& box) const
    {
        for (const Plane& p : _planes)
        {
            float v = p[3];
            for (size_t i = 0; i < 3; ++i)
                v += p[i] * (p[i] >= 0.0f ? box.getMax()[i] : box.getMin()[i]);
            if (v < 0.0f)
                return false;
        }
        return true;
    }

    bool operator==(const Frustum& o) const { return _mv == o._mv && _proj == o._proj; }
    bool operator!=(const Frustum& o) const { return !(*this == o); }

private:
    Matrix4f _mv, _proj, _invMV, _invProj;
    Vector3f _eye, _dir;
    float _left = 0, _right = 0, _bottom = 0, _top = 0, _near = 0, _far = 0;
    Plane _planes[6];
};
} // namespace livre

#endif
