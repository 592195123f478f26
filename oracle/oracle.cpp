/*
 * Livre hot-path oracle (CPU restatement). TEST INFRASTRUCTURE ONLY: the
 * product never links or calls it. Built with -ffp-contract=off so every
 * float expression below is a sequence of single IEEE round-to-nearest
 * operations in source order; where the kernel uses a fused multiply-add the
 * oracle calls std::fmaf (correctly rounded) at the same point.
 *
 * Reference files restated (paths inside the BlueBrain/Livre project):
 *  - livre/data/NodeId.cpp:23-163, livre/data/types.h:80-93
 *  - livre/data/DataSourcePlugin.cpp:40-95, livre/data/LODNode.cpp:30-64
 *  - livre/data/Frustum.cpp:24-76 (vmmlib Frustumf / FrustumCullerf math,
 *    third-party vmmlib f4b3706 is not vendored: restated from the published
 *    Gribb-Hartmann plane extraction and p-vertex box test)
 *  - livre/data/DFSTraversal.cpp:29-76, livre/data/SelectVisibles.cpp:45-131
 *  - livre/core/render/TransferFunction1D.cpp:56-107
 *  - livre/eq/render/shaders/fragRayCast.glsl:72-207,
 *    livre/eq/render/RayCastRenderer.cpp:57-81,213-386,503-571
 */
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace
{
/* ---------------------------------------------------------------- NodeId */
inline uint32_t nid_level(uint64_t id) { return uint32_t(id & 0xFu); }
inline uint32_t nid_x(uint64_t id) { return uint32_t((id >> 4) & 0x3FFFu); }
inline uint32_t nid_y(uint64_t id) { return uint32_t((id >> 18) & 0x3FFFu); }
inline uint32_t nid_z(uint64_t id) { return uint32_t((id >> 32) & 0x3FFFu); }
inline uint32_t nid_t(uint64_t id) { return uint32_t(id >> 46); }
inline uint64_t nid_make(uint32_t level, uint32_t x, uint32_t y, uint32_t z,
                         uint32_t t)
{
    return uint64_t(level & 0xFu) | (uint64_t(x & 0x3FFFu) << 4) |
           (uint64_t(y & 0x3FFFu) << 18) | (uint64_t(z & 0x3FFFu) << 32) |
           (uint64_t(t & 0x3FFFFu) << 46);
}

/* ---------------------------------------------------------- matrix math */
/* Column-major 4x4: element (row r, column c) is m[c * 4 + r]. */
inline float M(const float* m, int r, int c) { return m[c * 4 + r]; }

void mat_mul(const float* a, const float* b, float* out)
{
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c)
        {
            float acc = 0.0f;
            for (int k = 0; k < 4; ++k)
                acc = acc + M(a, r, k) * M(b, k, c);
            out[c * 4 + r] = acc;
        }
}

/* Inverse by Laplace expansion along the first two rows (2x2 minors). */
bool mat_inverse(const float* m, float* inv)
{
    const float m00 = M(m, 0, 0), m01 = M(m, 0, 1), m02 = M(m, 0, 2),
                m03 = M(m, 0, 3);
    const float m10 = M(m, 1, 0), m11 = M(m, 1, 1), m12 = M(m, 1, 2),
                m13 = M(m, 1, 3);
    const float m20 = M(m, 2, 0), m21 = M(m, 2, 1), m22 = M(m, 2, 2),
                m23 = M(m, 2, 3);
    const float m30 = M(m, 3, 0), m31 = M(m, 3, 1), m32 = M(m, 3, 2),
                m33 = M(m, 3, 3);
    const float s0 = m00 * m11 - m10 * m01;
    const float s1 = m00 * m12 - m10 * m02;
    const float s2 = m00 * m13 - m10 * m03;
    const float s3 = m01 * m12 - m11 * m02;
    const float s4 = m01 * m13 - m11 * m03;
    const float s5 = m02 * m13 - m12 * m03;
    const float c5 = m22 * m33 - m32 * m23;
    const float c4 = m21 * m33 - m31 * m23;
    const float c3 = m21 * m32 - m31 * m22;
    const float c2 = m20 * m33 - m30 * m23;
    const float c1 = m20 * m32 - m30 * m22;
    const float c0 = m20 * m31 - m30 * m21;
    const float det =
        s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    if (det == 0.0f || !std::isfinite(det))
        return false;
    const float id = 1.0f / det;
    float r[4][4];
    r[0][0] = (m11 * c5 - m12 * c4 + m13 * c3) * id;
    r[0][1] = (-m01 * c5 + m02 * c4 - m03 * c3) * id;
    r[0][2] = (m31 * s5 - m32 * s4 + m33 * s3) * id;
    r[0][3] = (-m21 * s5 + m22 * s4 - m23 * s3) * id;
    r[1][0] = (-m10 * c5 + m12 * c2 - m13 * c1) * id;
    r[1][1] = (m00 * c5 - m02 * c2 + m03 * c1) * id;
    r[1][2] = (-m30 * s5 + m32 * s2 - m33 * s1) * id;
    r[1][3] = (m20 * s5 - m22 * s2 + m23 * s1) * id;
    r[2][0] = (m10 * c4 - m11 * c2 + m13 * c0) * id;
    r[2][1] = (-m00 * c4 + m01 * c2 - m03 * c0) * id;
    r[2][2] = (m30 * s4 - m31 * s2 + m33 * s0) * id;
    r[2][3] = (-m20 * s4 + m21 * s2 - m23 * s0) * id;
    r[3][0] = (-m10 * c3 + m11 * c1 - m12 * c0) * id;
    r[3][1] = (m00 * c3 - m01 * c1 + m02 * c0) * id;
    r[3][2] = (-m30 * s3 + m31 * s1 - m32 * s0) * id;
    r[3][3] = (m20 * s3 - m21 * s1 + m22 * s0) * id;
    for (int rr = 0; rr < 4; ++rr)
        for (int cc = 0; cc < 4; ++cc)
            inv[cc * 4 + rr] = r[rr][cc];
    return true;
}

/* plane . (p, 1) summed left to right: ((a*x + b*y) + c*z) + d */
inline float plane_dot(const float* pl, const float* p)
{
    return pl[0] * p[0] + pl[1] * p[1] + pl[2] * p[2] + pl[3];
}

struct Frustum
{
    or_frustum f;
};

/* Box outside one plane: the corner farthest along the normal (p-vertex) is
 * on the negative side. */
inline bool box_outside_plane(const float* pl, const float* bmin,
                              const float* bmax)
{
    float pv[3];
    for (int i = 0; i < 3; ++i)
        pv[i] = pl[i] >= 0.0f ? bmax[i] : bmin[i];
    return plane_dot(pl, pv) < 0.0f;
}

struct Volume
{
    or_volume v;
    uint32_t block[3];
};

inline void world_box(const or_volume& v, uint64_t id, float* bmin,
                      float* bmax)
{
    const uint32_t level = nid_level(id);
    uint32_t bricks[3];
    for (int i = 0; i < 3; ++i)
        bricks[i] = v.root_blocks[i] << level;
    /* vmml find_max_index: first index of the maximum */
    int idx = 0;
    for (int i = 1; i < 3; ++i)
        if (bricks[i] > bricks[idx])
            idx = i;
    const float denom = float(bricks[idx]);
    const uint32_t pos[3] = {nid_x(id), nid_y(id), nid_z(id)};
    for (int i = 0; i < 3; ++i)
    {
        const float cmin = float(int32_t(pos[i])) / denom;
        const float cmax = float(int32_t(pos[i] + 1u)) / denom;
        const float half = v.world_size[i] * 0.5f;
        bmin[i] = cmin * v.world_size[i] - half;
        bmax[i] = cmax * v.world_size[i] - half;
    }
}

/* ------------------------------------------------------ LOD selection */
struct Selector
{
    const or_volume* vol;
    or_frustum fr;
    uint32_t H;
    float sse;
    uint32_t minLOD, maxLOD;
    const float* clip;
    uint32_t nclip;
    std::vector<uint64_t> visibles;
    uint64_t visited = 0;

    bool in_frustum(const float* bmin, const float* bmax) const
    {
        for (int p = 0; p < 6; ++p)
            if (box_outside_plane(fr.planes[p], bmin, bmax))
                return false;
        return true;
    }

    bool clip_outside(const float* bmin, const float* bmax) const
    {
        for (uint32_t p = 0; p < nclip; ++p)
            if (box_outside_plane(clip + 4 * p, bmin, bmax))
                return true;
        return false;
    }

    /* SelectVisibles.cpp:45-64 */
    bool lod_visible(const float* coord, float wspv) const
    {
        const float wspp = (fr.top - fr.bottom) / float(H);
        const float ppv = wspv / wspp;
        const float distance = std::fabs(plane_dot(fr.planes[4], coord));
        const float n = fr.nearp;
        const float ppvd = ppv * n / (n + distance);
        return ppvd <= sse;
    }

    /* SelectVisibles.cpp:66-107; returns true to descend */
    bool visit(uint64_t id)
    {
        ++visited;
        float bmin[3], bmax[3];
        world_box(*vol, id, bmin, bmax);
        if (!in_frustum(bmin, bmax) || clip_outside(bmin, bmax))
            return false;

        const float* np = fr.planes[4];
        float vmin[3], vmax[3];
        for (int i = 0; i < 3; ++i)
        {
            if (np[i] >= 0.0f)
            {
                vmin[i] = bmin[i];
                vmax[i] = bmax[i];
            }
            else
            {
                vmin[i] = bmax[i];
                vmax[i] = bmin[i];
            }
        }
        if (plane_dot(np, vmin) < 0.0f || plane_dot(np, vmax) < 0.0f)
        {
            for (int i = 0; i < 3; ++i)
                vmin[i] = fr.eye[i] - fr.dir[i] * fr.nearp;
        }
        float wspv = 0.0f;
        for (int i = 0; i < 3; ++i)
        {
            const uint32_t bs = vol->max_block[i] - 2u * vol->overlap[i];
            const float w = (bmax[i] - bmin[i]) / float(bs);
            wspv = (i == 0 || w < wspv) ? w : wspv;
        }
        bool visible = lod_visible(vmin, wspv);
        const uint32_t level = nid_level(id);
        visible = (visible && level >= minLOD) || level == maxLOD ||
                  level == vol->depth - 1u;
        if (visible)
            visibles.push_back(id);
        return !visible;
    }

    void traverse(uint64_t id, uint32_t depth)
    {
        if (!visit(id))
            return;
        if (depth == 1)
            return;
        uint64_t ch[8];
        or_node_children(id, ch);
        for (int i = 0; i < 8; ++i)
            traverse(ch[i], depth - 1);
    }
};

/* ------------------------------------------------------------ blobs */
inline uint64_t splitmix_next(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t splitmix_mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline float u01(uint64_t r) { return float(r >> 40) * (1.0f / 16777216.0f); }

struct Blob
{
    float cx, cy, cz, inv2s2, cut2, amp;
};

std::vector<Blob> make_blobs(const or_volume& v, const or_blob_params& bp)
{
    std::vector<Blob> blobs(bp.n_blobs);
    uint64_t s = bp.seed;
    for (uint32_t i = 0; i < bp.n_blobs; ++i)
    {
        Blob& b = blobs[i];
        b.cx = u01(splitmix_next(s)) * float(v.voxels[0]);
        b.cy = u01(splitmix_next(s)) * float(v.voxels[1]);
        b.cz = u01(splitmix_next(s)) * float(v.voxels[2]);
        const float sigma = 8.0f + 24.0f * u01(splitmix_next(s));
        b.amp = 0.3f + 0.7f * u01(splitmix_next(s));
        b.inv2s2 = 1.0f / (2.0f * sigma * sigma);
        const float c = 6.0f * sigma;
        b.cut2 = c * c;
    }
    return blobs;
}

inline float blob_sum(const std::vector<Blob>& blobs, const uint32_t* cand,
                      uint32_t ncand, float x, float y, float z)
{
    float acc = 0.0f;
    for (uint32_t j = 0; j < ncand; ++j)
    {
        const Blob& b = blobs[cand[j]];
        const float dx = x - b.cx, dy = y - b.cy, dz = z - b.cz;
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 < b.cut2)
            acc = acc + b.amp * or_exp_neg(-(d2 * b.inv2s2));
    }
    return acc;
}

uint64_t noise_key(uint64_t seed, uint32_t level, uint32_t x, uint32_t y,
                   uint32_t z)
{
    const uint64_t P = 0x100000001B3ull;
    uint64_t k = seed;
    k = k * P + level;
    k = k * P + x;
    k = k * P + y;
    k = k * P + z;
    return splitmix_mix(k);
}

/* -------------------------------------------------------------- raycast */
struct RenderSet
{
    const or_volume* vol;
    uint32_t dtype;
    uint32_t N[3];     /* slot voxels per axis */
    uint32_t B[3];     /* block size */
    uint32_t O[3];     /* overlap */
    size_t brickVoxels;
    const uint8_t* bricks;
    std::vector<uint64_t> ids;
    uint32_t Lf;       /* finest level */
    uint32_t dims[3];  /* leaf grid cells per axis */
    std::vector<int32_t> leaf; /* index into ids, -1 empty */
    bool quant_weights = false; /* OR_QUANT_WEIGHTS */

    double voxel(uint32_t brick, int x, int y, int z) const
    {
        x = std::min(std::max(x, 0), int(N[0]) - 1);
        y = std::min(std::max(y, 0), int(N[1]) - 1);
        z = std::min(std::max(z, 0), int(N[2]) - 1);
        const size_t k = brick * brickVoxels +
                         (size_t(z) * N[1] + size_t(y)) * N[0] + size_t(x);
        /* lv_dtype codes: 0 float, 1 uint8, 2 uint16, 3 uint32, 4 int8,
         * 5 int16, 6 int32 (the voxel value as the GL shader's texel) */
        switch (dtype)
        {
        case 0: return double(reinterpret_cast<const float*>(bricks)[k]);
        case 2: return double(reinterpret_cast<const uint16_t*>(bricks)[k]);
        case 3: return double(reinterpret_cast<const uint32_t*>(bricks)[k]);
        case 4: return double(reinterpret_cast<const int8_t*>(bricks)[k]);
        case 5: return double(reinterpret_cast<const int16_t*>(bricks)[k]);
        case 6: return double(reinterpret_cast<const int32_t*>(bricks)[k]);
        default: return double(bricks[k]);
        }
    }

    /* Per-ray mode: s = FP32 slot coordinate (nearest: the local position;
     * trilinear: local position - 0.5, texel centres on integers), computed
     * with the same FMA chain as the kernel; taps clamp to the brick
     * (GL_CLAMP_TO_EDGE) and the weights are evaluated in double. */
    double sample_f(uint32_t brick, const float s[3], uint32_t filter) const
    {
        if (filter == 0)
            return voxel(brick, int(std::floor(s[0])), int(std::floor(s[1])),
                         int(std::floor(s[2])));
        double f[3];
        int i0[3];
        for (int a = 0; a < 3; ++a)
        {
            const float fl = std::floor(s[a]);
            i0[a] = int(fl);
            f[a] = double(s[a] - fl);
            if (quant_weights) /* round to the nearest 1/256 */
                f[a] = std::nearbyint(f[a] * 256.0) / 256.0;
        }
        double c[2][2][2];
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx)
                    c[dz][dy][dx] = voxel(brick, i0[0] + dx, i0[1] + dy, i0[2] + dz);
        double cy[2][2], cz[2];
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                cy[dz][dy] = c[dz][dy][0] + (c[dz][dy][1] - c[dz][dy][0]) * f[0];
        for (int dz = 0; dz < 2; ++dz)
            cz[dz] = cy[dz][0] + (cy[dz][1] - cy[dz][0]) * f[1];
        return cz[0] + (cz[1] - cz[0]) * f[2];
    }

    /* sv: continuous voxel coordinate inside the slot (texel centres at +0.5) */
    double sample(uint32_t brick, const double sv[3], uint32_t filter) const
    {
        if (filter == 0)
            return voxel(brick, int(std::floor(sv[0])), int(std::floor(sv[1])),
                         int(std::floor(sv[2])));
        double f[3];
        int i0[3];
        for (int a = 0; a < 3; ++a)
        {
            const double s = sv[a] - 0.5;
            const double fl = std::floor(s);
            i0[a] = int(fl);
            f[a] = s - fl;
        }
        double c[2][2][2];
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx)
                    c[dz][dy][dx] =
                        voxel(brick, i0[0] + dx, i0[1] + dy, i0[2] + dz);
        double cy[2][2], cz[2];
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                cy[dz][dy] = c[dz][dy][0] + (c[dz][dy][1] - c[dz][dy][0]) * f[0];
        for (int dz = 0; dz < 2; ++dz)
            cz[dz] = cy[dz][0] + (cy[dz][1] - cy[dz][0]) * f[1];
        return cz[0] + (cz[1] - cz[0]) * f[2];
    }
};

struct Shade
{
    const float* tf;
    uint32_t tfn;
    double mul, add, ac, early;

    /* GL_LINEAR + CLAMP_TO_EDGE lookup of an N-texel 1D texture */
    void tf_lookup(double d, double rgba[4]) const
    {
        const double s = d * double(tfn) - 0.5;
        const double fl = std::floor(s);
        const double f = s - fl;
        long i0 = long(fl), i1 = i0 + 1;
        i0 = std::min(std::max(i0, 0L), long(tfn) - 1);
        i1 = std::min(std::max(i1, 0L), long(tfn) - 1);
        for (int c = 0; c < 4; ++c)
            rgba[c] = double(tf[i0 * 4 + c]) * (1.0 - f) +
                      double(tf[i1 * 4 + c]) * f;
    }

    /* fragRayCast.glsl:103-111 */
    void composite(const double src[4], double dst[4]) const
    {
        const double alpha =
            1.0 - std::pow(1.0 - std::min(src[3], 1.0 - 1.0 / 256.0), ac);
        for (int c = 0; c < 3; ++c)
            dst[c] += src[c] * alpha * (1.0 - dst[3]);
        dst[3] += alpha * (1.0 - dst[3]);
    }
};

/* FP32 ray set-up shared by the per-ray mode; every op is IEEE single. */
struct Ray32
{
    float eye[3], dir[3];
    float tNearPlane;
    float t0, t1; /* global box */
};

void ray_setup32(const or_frustum& fr, const float* gmin, const float* gmax,
                 uint32_t W, uint32_t H, uint32_t px, uint32_t py, Ray32& r)
{
    const float nx = (float(px) + 0.5f) * 2.0f / float(W) - 1.0f;
    const float ny = (float(py) + 0.5f) * 2.0f / float(H) - 1.0f;
    const float v[4] = {nx, ny, -1.0f, 1.0f};
    float e[4];
    for (int i = 0; i < 4; ++i)
        e[i] = M(fr.inv_p, i, 0) * v[0] + M(fr.inv_p, i, 1) * v[1] +
               M(fr.inv_p, i, 2) * v[2] + M(fr.inv_p, i, 3) * v[3];
    const float ep[3] = {e[0] / e[3], e[1] / e[3], e[2] / e[3]};
    float pw[3], d[3];
    for (int i = 0; i < 3; ++i)
        pw[i] = M(fr.inv_mv, i, 0) * ep[0] + M(fr.inv_mv, i, 1) * ep[1] +
                M(fr.inv_mv, i, 2) * ep[2] + M(fr.inv_mv, i, 3);
    for (int i = 0; i < 3; ++i)
    {
        r.eye[i] = fr.eye[i];
        d[i] = pw[i] - fr.eye[i];
    }
    const float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for (int i = 0; i < 3; ++i)
        r.dir[i] = d[i] / len;
    const float lenE =
        std::sqrt(ep[0] * ep[0] + ep[1] * ep[1] + ep[2] * ep[2]);
    const float nz = ep[2] / lenE;
    r.tNearPlane = -fr.nearp / nz;

    float tmin[3], tmax[3];
    for (int i = 0; i < 3; ++i)
    {
        const float di = r.dir[i] == 0.0f ? 1e-10f : r.dir[i];
        const float inv = 1.0f / di;
        const float tb = inv * (gmin[i] - r.eye[i]);
        const float tt = inv * (gmax[i] - r.eye[i]);
        tmin[i] = std::min(tt, tb);
        tmax[i] = std::max(tt, tb);
    }
    r.t0 = std::max(std::max(tmin[0], tmin[1]), std::max(tmin[0], tmin[2]));
    r.t1 = std::min(std::min(tmax[0], tmax[1]), std::min(tmax[0], tmax[2]));
}

/* Whether a brick's entry parameter is the previous brick's exit: the ray
 * crossed a face the two bricks share (diagnostics of or_raycast_px). */
bool t_entry_face(double prev_exit, double entry)
{
    return std::fabs(entry - prev_exit) <= 1e-9 * std::max(1.0, std::fabs(entry));
}

/* double-precision slab test of fragRayCast.glsl:79-101 */
bool intersect64(const double* o, const double* d, const double* bmin,
                 const double* bmax, double& t0, double& t1)
{
    double tmin[3], tmax[3];
    for (int i = 0; i < 3; ++i)
    {
        const double di = d[i] == 0.0 ? 1e-10 : d[i];
        const double inv = 1.0 / di;
        const double tb = inv * (bmin[i] - o[i]);
        const double tt = inv * (bmax[i] - o[i]);
        tmin[i] = std::min(tt, tb);
        tmax[i] = std::max(tt, tb);
    }
    t0 = std::max(std::max(tmin[0], tmin[1]), std::max(tmin[0], tmin[2]));
    t1 = std::min(std::min(tmax[0], tmax[1]), std::min(tmax[0], tmax[2]));
    return t0 <= t1;
}

} // namespace

extern "C" {

int or_fill_regular_volume_info(or_volume* v)
{
    uint32_t maxv = std::max(v->voxels[0], std::max(v->voxels[1], v->voxels[2]));
    if (maxv == 0)
        return -1;
    v->wspv = 1.0f / float(maxv);
    for (int i = 0; i < 3; ++i)
        v->world_size[i] = float(v->voxels[i]) * v->wspv;
    uint32_t bs[3], nb[3], lod[3];
    for (int i = 0; i < 3; ++i)
    {
        if (v->max_block[i] <= 2u * v->overlap[i])
            return -1;
        bs[i] = v->max_block[i] - 2u * v->overlap[i];
        nb[i] = uint32_t(std::ceil(float(v->voxels[i]) / float(bs[i])));
        lod[i] = uint32_t(std::ceil(std::log2(double(nb[i]))));
    }
    const uint32_t depth = std::min(lod[0], std::min(lod[1], lod[2]));
    for (int i = 0; i < 3; ++i)
        v->root_blocks[i] =
            uint32_t(std::ceil(float(v->voxels[i] >> depth) / float(bs[i])));
    v->depth = depth + 1;
    return 0;
}

void or_node_world_box(const or_volume* vol, uint64_t id, float box[6])
{
    world_box(*vol, id, box, box + 3);
}

void or_node_children(uint64_t id, uint64_t out[8])
{
    const uint32_t l = nid_level(id), t = nid_t(id);
    const uint32_t x = nid_x(id) * 2, y = nid_y(id) * 2, z = nid_z(id) * 2;
    int k = 0;
    for (uint32_t i = 0; i < 2; ++i)
        for (uint32_t j = 0; j < 2; ++j)
            for (uint32_t m = 0; m < 2; ++m)
                out[k++] = nid_make(l + 1, x + i, y + j, z + m, t);
}

int or_frustum_setup(const float* mv, const float* p, or_frustum* f)
{
    if (!mat_inverse(mv, f->inv_mv) || !mat_inverse(p, f->inv_p))
        return -1;
    /* vmml Frustumf(projection) limits */
    const float p22 = M(p, 2, 2), p23 = M(p, 2, 3);
    f->nearp = p23 / (p22 - 1.0f);
    f->farp = p23 / (p22 + 1.0f);
    f->bottom = f->nearp * (M(p, 1, 2) - 1.0f) / M(p, 1, 1);
    f->top = f->nearp * (M(p, 1, 2) + 1.0f) / M(p, 1, 1);
    f->left = f->nearp * (M(p, 0, 2) - 1.0f) / M(p, 0, 0);
    f->right = f->nearp * (M(p, 0, 2) + 1.0f) / M(p, 0, 0);

    /* FrustumCuller(P * MV): Gribb-Hartmann planes, normalised */
    float pm[16];
    mat_mul(p, mv, pm);
    float row[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c)
            row[r][c] = M(pm, r, c);
    for (int c = 0; c < 4; ++c)
    {
        f->planes[0][c] = row[3][c] + row[0][c];
        f->planes[1][c] = row[3][c] - row[0][c];
        f->planes[2][c] = row[3][c] + row[1][c];
        f->planes[3][c] = row[3][c] - row[1][c];
        f->planes[4][c] = row[3][c] + row[2][c];
        f->planes[5][c] = row[3][c] - row[2][c];
    }
    for (int pl = 0; pl < 6; ++pl)
    {
        float* q = f->planes[pl];
        const float len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
        const float inv = float(1.0 / double(len));
        for (int c = 0; c < 4; ++c)
            q[c] = q[c] * inv;
    }
    for (int i = 0; i < 3; ++i)
    {
        f->eye[i] = M(f->inv_mv, i, 3);
        f->dir[i] = M(f->inv_mv, i, 2);
    }
    return 0;
}

int or_select_visible(const or_volume* vol, const float* mv, const float* proj,
                      uint32_t window_height, float sse, uint32_t min_lod,
                      uint32_t max_lod, const float* range,
                      const float* clip_planes, uint32_t n_clip,
                      uint32_t time_step, uint64_t* out, uint32_t capacity,
                      uint32_t* n_out, uint64_t* n_visited)
{
    Selector s;
    s.vol = vol;
    if (or_frustum_setup(mv, proj, &s.fr) != 0)
        return -2;
    s.H = window_height;
    s.sse = sse;
    s.minLOD = min_lod;
    s.maxLOD = max_lod;
    s.clip = clip_planes;
    s.nclip = n_clip;
    for (uint32_t x = 0; x < vol->root_blocks[0]; ++x)
        for (uint32_t y = 0; y < vol->root_blocks[1]; ++y)
            for (uint32_t z = 0; z < vol->root_blocks[2]; ++z)
                s.traverse(nid_make(0, x, y, z, time_step), vol->depth);
    /* visitPost range slice (SelectVisibles.cpp:110-131) */
    const size_t n = s.visibles.size();
    const size_t start = size_t(range[0] * float(n));
    const size_t end = size_t(range[1] * float(n));
    uint32_t k = 0;
    int rc = 0;
    for (size_t i = 0; i < n; ++i)
    {
        if (i >= start && i < end)
        {
            if (k < capacity)
                out[k] = s.visibles[i];
            else
                rc = -1;
            ++k;
        }
    }
    *n_out = k;
    if (n_visited)
        *n_visited = s.visited;
    return rc;
}

void or_default_tf(float* rgba)
{
    const float color1[3] = {0.0f, 1.0f, 1.0f};
    const float color2[3] = {1.0f, 0.0f, 1.0f};
    const float alpha1 = 0.39f, alpha2 = 0.03f;
    const float density1 = 127.f, density2 = 255.f;
    float colorDiff[3];
    for (int c = 0; c < 3; ++c)
        colorDiff[c] = color2[c] - color1[c];
    const float alphaDiff = alpha2 - alpha1;
    for (uint32_t i = 0; i < 256; ++i)
    {
        float v[4] = {0.f, 0.f, 0.f, 0.f};
        if (i > 0 && float(i) <= density1)
        {
            for (int c = 0; c < 3; ++c)
                v[c] = color1[c];
            v[3] = alpha1 * (float(i) / density1);
        }
        else if (i > 0)
        {
            const float w = (float(i) - density1 + 1.f) /
                            (density2 - density1 + 1.f);
            for (int c = 0; c < 3; ++c)
                v[c] = w * colorDiff[c] + color1[c];
            v[3] = w * alphaDiff + alpha1;
        }
        for (int c = 0; c < 4; ++c)
            rgba[i * 4 + c] = v[c];
    }
}

void or_tf_lut(const float* rgba, uint32_t n, uint8_t* lut)
{
    for (uint32_t i = 0; i < n * 4; ++i)
        lut[i] = uint8_t(rgba[i] * 255.f);
}

/* exp(x) for x <= 0 as 2^(x*log2 e): n = floor, f = fraction, 2^f by the
 * degree-7 Taylor series of e^(f ln 2) in Horner form, scaled by 2^n. */
float or_exp_neg(float x)
{
    if (x < -80.0f)
        return 0.0f;
    const float y = x * 1.44269504f;
    const float n = std::floor(y);
    const float f = y - n;
    const float c1 = 0.693147182f, c2 = 0.240226507f, c3 = 0.0555041087f,
                c4 = 0.00961812911f, c5 = 0.00133335581f,
                c6 = 0.000154035304f, c7 = 1.52527338e-05f;
    float p = c7;
    p = p * f + c6;
    p = p * f + c5;
    p = p * f + c4;
    p = p * f + c3;
    p = p * f + c2;
    p = p * f + c1;
    p = p * f + 1.0f;
    return std::ldexp(p, int(n));
}

float or_blob_value(const or_volume* vol, const or_blob_params* bp, float x,
                    float y, float z)
{
    const std::vector<Blob> blobs = make_blobs(*vol, *bp);
    std::vector<uint32_t> all(blobs.size());
    for (uint32_t i = 0; i < all.size(); ++i)
        all[i] = i;
    return blob_sum(blobs, all.data(), uint32_t(all.size()), x, y, z);
}

int or_blob_brick(const or_volume* vol, const or_blob_params* bp,
                  uint64_t id, void* out)
{
    const std::vector<Blob> blobs = make_blobs(*vol, *bp);
    const uint32_t level = nid_level(id);
    if (level >= vol->depth)
        return -1;
    const uint32_t shift = vol->depth - 1u - level;
    const uint32_t s = 1u << shift;
    const uint32_t pos[3] = {nid_x(id), nid_y(id), nid_z(id)};
    uint32_t N[3], B[3], VL[3];
    int32_t base[3];
    for (int a = 0; a < 3; ++a)
    {
        N[a] = vol->max_block[a];
        B[a] = N[a] - 2u * vol->overlap[a];
        VL[a] = (vol->voxels[a] + s - 1u) >> shift;
        base[a] = int32_t(pos[a] * B[a]) - int32_t(vol->overlap[a]);
    }
    /* candidate blobs: cut-off sphere touches the brick's sample box */
    std::vector<uint32_t> cand;
    for (uint32_t i = 0; i < blobs.size(); ++i)
    {
        const Blob& b = blobs[i];
        const float c[3] = {b.cx, b.cy, b.cz};
        double d2 = 0.0;
        for (int a = 0; a < 3; ++a)
        {
            int32_t lo = std::max(base[a], 0);
            int32_t hi = std::min(base[a] + int32_t(N[a]) - 1, int32_t(VL[a]) - 1);
            lo = std::min(lo, int32_t(VL[a]) - 1);
            hi = std::max(hi, 0);
            const double flo = (double(lo) + 0.5) * s - 1.0;
            const double fhi = (double(hi) + 0.5) * s + 1.0;
            double dd = 0.0;
            if (c[a] < flo)
                dd = flo - c[a];
            else if (c[a] > fhi)
                dd = c[a] - fhi;
            d2 += dd * dd;
        }
        if (d2 < double(b.cut2) * 1.01 + 1.0)
            cand.push_back(i);
    }
    const float fs = float(s);
    for (uint32_t k = 0; k < N[2]; ++k)
        for (uint32_t j = 0; j < N[1]; ++j)
            for (uint32_t i = 0; i < N[0]; ++i)
            {
                const uint32_t g[3] = {
                    uint32_t(std::min(std::max(base[0] + int32_t(i), 0), int32_t(VL[0]) - 1)),
                    uint32_t(std::min(std::max(base[1] + int32_t(j), 0), int32_t(VL[1]) - 1)),
                    uint32_t(std::min(std::max(base[2] + int32_t(k), 0), int32_t(VL[2]) - 1))};
                const float x = (float(g[0]) + 0.5f) * fs;
                const float y = (float(g[1]) + 0.5f) * fs;
                const float z = (float(g[2]) + 0.5f) * fs;
                float v = blob_sum(blobs, cand.data(), uint32_t(cand.size()), x, y, z);
                v = std::min(std::max(v, 0.0f), 1.0f);
                int32_t noise = 0;
                if (bp->noise)
                {
                    const uint64_t h = noise_key(bp->seed, level, g[0], g[1], g[2]);
                    noise = int32_t(h % (2u * bp->noise + 1u)) - int32_t(bp->noise);
                }
                const size_t idx = (size_t(k) * N[1] + j) * N[0] + i;
                if (bp->dtype == 2)
                {
                    int32_t q = int32_t(std::floor(v * 65535.0f + 0.5f)) + noise * 257;
                    q = std::min(std::max(q, 0), 65535);
                    static_cast<uint16_t*>(out)[idx] = uint16_t(q);
                }
                else
                {
                    int32_t q = int32_t(std::floor(v * 255.0f + 0.5f)) + noise;
                    q = std::min(std::max(q, 0), 255);
                    static_cast<uint8_t*>(out)[idx] = uint8_t(q);
                }
            }
    return 0;
}

/* ---- fBm over improved Perlin noise (the 8192^3 uint16 workload's
 * synthetic input). Published algorithm: quintic fade 6t^5 - 15t^4 + 10t^3,
 * gradients (+-1, +-1, 0) and permutations of it chosen by hash & 15 (with
 * 12..15 repeating four of them), trilinear blend of the eight corner dot
 * products. */
namespace
{
struct Perlin
{
    uint16_t perm[512];

    explicit Perlin(uint64_t seed)
    {
        for (uint32_t i = 0; i < 256; ++i)
            perm[i] = uint16_t(i);
        uint64_t state = seed;
        for (uint32_t i = 255; i > 0; --i)
        {
            state += 0x9E3779B97F4A7C15ull;
            uint64_t z = state;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z ^= z >> 31;
            const uint32_t j = uint32_t(z % (i + 1u));
            const uint16_t t = perm[i];
            perm[i] = perm[j];
            perm[j] = t;
        }
        for (uint32_t i = 0; i < 256; ++i)
            perm[256 + i] = perm[i];
    }

    static float smooth(float t)
    {
        const float inner = t * (t * 6.0f - 15.0f) + 10.0f;
        return t * t * t * inner;
    }
    static float mix(float w, float a, float b) { return a + w * (b - a); }
    static float corner(uint32_t h, float x, float y, float z)
    {
        switch (h & 15u)
        {
        case 0: return x + y;
        case 1: return -x + y;
        case 2: return x + -y;
        case 3: return -x + -y;
        case 4: return x + z;
        case 5: return -x + z;
        case 6: return x + -z;
        case 7: return -x + -z;
        case 8: return y + z;
        case 9: return -y + z;
        case 10: return y + -z;
        case 11: return -y + -z;
        case 12: return y + x;
        case 13: return -y + z;
        case 14: return y + -x;
        default: return -y + -z;
        }
    }

    float operator()(float x, float y, float z) const
    {
        const float xf = std::floor(x), yf = std::floor(y), zf = std::floor(z);
        const uint32_t xi = uint32_t(int32_t(xf)) & 255u, yi = uint32_t(int32_t(yf)) & 255u,
                       zi = uint32_t(int32_t(zf)) & 255u;
        const float dx = x - xf, dy = y - yf, dz = z - zf;
        const float u = smooth(dx), v = smooth(dy), w = smooth(dz);
        float c[2][2][2];
        for (uint32_t k = 0; k < 2; ++k)
            for (uint32_t j = 0; j < 2; ++j)
                for (uint32_t i = 0; i < 2; ++i)
                {
                    const uint32_t h = perm[perm[perm[xi + i] + yi + j] + zi + k];
                    c[k][j][i] = corner(h, i ? dx - 1.0f : dx, j ? dy - 1.0f : dy,
                                        k ? dz - 1.0f : dz);
                }
        const float y0 = mix(v, mix(u, c[0][0][0], c[0][0][1]), mix(u, c[0][1][0], c[0][1][1]));
        const float y1 = mix(v, mix(u, c[1][0][0], c[1][0][1]), mix(u, c[1][1][0], c[1][1][1]));
        return mix(w, y0, y1);
    }
};
} // namespace

float or_perlin(uint64_t seed, float x, float y, float z)
{
    return Perlin(seed)(x, y, z);
}

int or_fbm_brick(const or_volume* vol, const or_fbm_params* fp, uint64_t id, void* out)
{
    const uint32_t level = nid_level(id);
    if (level >= vol->depth || fp->octaves == 0)
        return -1;
    const Perlin noise(fp->seed);
    const uint32_t shift = vol->depth - 1u - level;
    const uint32_t s = 1u << shift;
    const uint32_t vmax = std::max(vol->voxels[0], std::max(vol->voxels[1], vol->voxels[2]));
    const float scale = float(s) * (fp->frequency / float(vmax));
    const uint32_t pos[3] = {nid_x(id), nid_y(id), nid_z(id)};
    const uint32_t* N = vol->max_block;
    int32_t base[3], last[3];
    for (int a = 0; a < 3; ++a)
    {
        base[a] = int32_t(pos[a] * (N[a] - 2u * vol->overlap[a])) - int32_t(vol->overlap[a]);
        last[a] = int32_t((vol->voxels[a] + s - 1u) >> shift) - 1;
    }
    const float top = fp->dtype == 2 ? 65535.0f : 255.0f;
    size_t idx = 0;
    for (uint32_t k = 0; k < N[2]; ++k)
        for (uint32_t j = 0; j < N[1]; ++j)
            for (uint32_t i = 0; i < N[0]; ++i, ++idx)
            {
                const uint32_t off[3] = {i, j, k};
                float p[3];
                for (int a = 0; a < 3; ++a)
                {
                    const int32_t g = std::min(std::max(base[a] + int32_t(off[a]), 0), last[a]);
                    p[a] = (float(g) + 0.5f) * scale;
                }
                float sum = 0.0f, amp = 1.0f, f = 1.0f;
                for (uint32_t o = 0; o < fp->octaves; ++o)
                {
                    sum = sum + amp * noise(p[0] * f, p[1] * f, p[2] * f);
                    amp = amp * fp->gain;
                    f = f * fp->lacunarity;
                }
                const float v = std::min(std::max(sum, -1.0f), 1.0f);
                const uint32_t q = uint32_t(std::floor((v + 1.0f) * 0.5f * top + 0.5f));
                if (fp->dtype == 2)
                    static_cast<uint16_t*>(out)[idx] = uint16_t(q);
                else
                    static_cast<uint8_t*>(out)[idx] = uint8_t(q);
            }
    return 0;
}

int or_raycast(const or_volume* vol, uint32_t dtype, const uint64_t* node_ids,
               uint32_t n_nodes, const void* bricks, const float* tf_rgba,
               uint32_t tf_n, const or_view* view, int mode, int n_threads,
               uint32_t row_begin, uint32_t row_end, double* out,
               uint64_t* n_samples_out)
{
    return or_raycast_px(vol, dtype, node_ids, n_nodes, bricks, tf_rgba, tf_n, view, mode,
                         n_threads, row_begin, row_end, out, n_samples_out, nullptr,
                         nullptr);
}

int or_raycast_px(const or_volume* vol, uint32_t dtype, const uint64_t* node_ids,
                  uint32_t n_nodes, const void* bricks, const float* tf_rgba,
                  uint32_t tf_n, const or_view* view, int mode, int n_threads,
                  uint32_t row_begin, uint32_t row_end, double* out,
                  uint64_t* n_samples_out, uint32_t* px_samples, uint8_t* px_flags)
{
    or_frustum fr;
    if (or_frustum_setup(view->mv, view->proj, &fr) != 0)
        return -2;
    if (view->n_samples == 0 || tf_n == 0)
        return -1;
    /* OR_ACCUMULATE: rays start from the colour in `out` (a later pass of a
     * multi-pass frame, RenderPipeline.cpp:92-158) */
    const bool accumulate = (mode & OR_ACCUMULATE) != 0;
    const int base_mode = mode & ~(OR_ACCUMULATE | OR_QUANT_WEIGHTS);
    RenderSet rs;
    rs.quant_weights = (mode & OR_QUANT_WEIGHTS) != 0;
    rs.vol = vol;
    rs.dtype = dtype;
    for (int a = 0; a < 3; ++a)
    {
        rs.N[a] = vol->max_block[a];
        rs.O[a] = vol->overlap[a];
        rs.B[a] = rs.N[a] - 2u * rs.O[a];
    }
    rs.brickVoxels = size_t(rs.N[0]) * rs.N[1] * rs.N[2];
    rs.bricks = static_cast<const uint8_t*>(bricks);
    rs.ids.assign(node_ids, node_ids + n_nodes);
    rs.Lf = vol->depth - 1u;
    for (int a = 0; a < 3; ++a)
        rs.dims[a] = vol->root_blocks[a] << rs.Lf;
    rs.leaf.assign(size_t(rs.dims[0]) * rs.dims[1] * rs.dims[2], -1);
    for (uint32_t n = 0; n < n_nodes; ++n)
    {
        const uint64_t id = node_ids[n];
        const uint32_t L = nid_level(id);
        if (L > rs.Lf)
            return -1;
        const uint32_t sh = rs.Lf - L;
        const uint32_t p[3] = {nid_x(id), nid_y(id), nid_z(id)};
        for (uint32_t z = p[2] << sh; z < (p[2] + 1) << sh && z < rs.dims[2]; ++z)
            for (uint32_t y = p[1] << sh; y < (p[1] + 1) << sh && y < rs.dims[1]; ++y)
                for (uint32_t x = p[0] << sh; x < (p[0] + 1) << sh && x < rs.dims[0]; ++x)
                {
                    int32_t& e = rs.leaf[(size_t(z) * rs.dims[1] + y) * rs.dims[0] + x];
                    if (e < 0 || nid_level(node_ids[e]) > L)
                        e = int32_t(n);
                }
    }

    Shade sh;
    sh.tf = tf_rgba;
    sh.tfn = tf_n;
    sh.mul = 1.0 / (double(view->range_hi) - double(view->range_lo));
    sh.add = -double(view->range_lo) /
             (double(view->range_hi) - double(view->range_lo));
    sh.ac = double(view->alpha_correction);
    sh.early = double(view->early_exit);

    float gmin[3], gmax[3], gscale[3], goff[3];
    uint32_t bm = std::max(rs.dims[0], std::max(rs.dims[1], rs.dims[2]));
    for (int a = 0; a < 3; ++a)
    {
        const float half = vol->world_size[a] / 2.0f;
        gmin[a] = -half;
        gmax[a] = half;
        gscale[a] = float(bm) / vol->world_size[a];
        goff[a] = half * gscale[a];
    }
    const float step = 1.0f / float(view->n_samples);
    const uint32_t W = view->width, H = view->height;
    if (row_end > H)
        row_end = H;

    /* shader-order brick list (RayCastRenderer.cpp:57-81, 153-159) */
    std::vector<uint32_t> order(n_nodes);
    std::vector<float> dist(n_nodes);
    for (uint32_t n = 0; n < n_nodes; ++n)
    {
        order[n] = n;
        float bmin[3], bmax[3];
        world_box(*vol, node_ids[n], bmin, bmax);
        float c[3];
        for (int a = 0; a < 3; ++a)
            c[a] = (bmin[a] + bmax[a]) * 0.5f;
        float e[3];
        for (int i = 0; i < 3; ++i)
            e[i] = M(view->mv, i, 0) * c[0] + M(view->mv, i, 1) * c[1] +
                   M(view->mv, i, 2) * c[2] + M(view->mv, i, 3);
        dist[n] = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    }
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return dist[a] < dist[b]; });

    std::atomic<uint32_t> next_row(row_begin);
    std::atomic<uint64_t> total_samples(0);

    auto per_ray = [&](uint32_t px, uint32_t py, double* dst, uint64_t& cnt) {
        if (dst[3] > sh.early) /* a later pass of an opaque ray */
            return;
        Ray32 r;
        ray_setup32(fr, gmin, gmax, W, H, px, py, r);
        if (!(r.t0 <= r.t1))
            return;
        const float tg = r.t0;
        float tlo = std::max(r.t0, r.tNearPlane);
        float thi = r.t1;
        for (uint32_t c = 0; c < view->n_clip; ++c)
        {
            const float* cp = view->clip[c];
            float rn = r.dir[0] * cp[0] + r.dir[1] * cp[1] + r.dir[2] * cp[2];
            if (rn == 0.0f)
                rn = 1e-10f;
            const float ne = cp[0] * r.eye[0] + cp[1] * r.eye[1] + cp[2] * r.eye[2];
            const float t = -(ne + cp[3]) / rn;
            if (rn > 0.0f)
                tlo = std::max(tlo, t);
            else
                thi = std::min(thi, t);
        }
        if (!(tlo <= thi))
            return;
        int64_t k = 0;
        if (tlo > tg)
            k = int64_t(std::ceil((tlo - tg) / step));
        const float half_texel = view->filter ? 0.5f : 0.0f;
        for (;; ++k)
        {
            /* single-rounding fused multiply-adds, as the kernel */
            const float t = std::fmaf(float(k), step, tg);
            if (!(t < thi))
                break;
            float f[3];
            int32_t cell[3];
            bool inside = true;
            for (int a = 0; a < 3; ++a)
            {
                const float p = std::fmaf(r.dir[a], t, r.eye[a]);
                f[a] = std::fmaf(p, gscale[a], goff[a]);
                /* t in [tnearGlobal, tfarGlobal): the sample is in the
                 * volume's box; a cell index rounded one past the box's face
                 * (a sample on the entry or exit face, taken by the shader at
                 * tnear = tnearGlobal, fragRayCast.glsl:142-147) is the face
                 * cell. The high face is the box's only on the axes with the
                 * most cells (node boxes: LODNode.cpp:30-64). */
                float fl = std::max(std::floor(f[a]), 0.0f);
                if (rs.dims[a] == bm)
                    fl = std::min(fl, float(rs.dims[a] - 1u));
                if (!(fl >= 0.0f) || !(fl < float(rs.dims[a])))
                    inside = false;
                cell[a] = inside ? int32_t(fl) : 0;
            }
            if (!inside)
                continue;
            const int32_t e =
                rs.leaf[(size_t(cell[2]) * rs.dims[1] + cell[1]) * rs.dims[0] + cell[0]];
            if (e < 0)
                continue;
            const uint64_t id = rs.ids[e];
            const uint32_t L = nid_level(id);
            const uint32_t shf = rs.Lf - L;
            const uint32_t P[3] = {nid_x(id), nid_y(id), nid_z(id)};
            float sc[3];
            for (int a = 0; a < 3; ++a)
            {
                const float vs = float(rs.B[a]) / float(1u << shf);
                const float off =
                    (float(rs.O[a]) - float(P[a] * rs.B[a])) - half_texel;
                sc[a] = std::fmaf(f[a], vs, off);
            }
            const double val = rs.sample_f(uint32_t(e), sc, view->filter);
            const double dens = val * sh.mul + sh.add;
            double src[4];
            sh.tf_lookup(dens, src);
            sh.composite(src, dst);
            ++cnt;
            if (dst[3] > sh.early)
                break;
        }
    };

    auto shader = [&](uint32_t px, uint32_t py, double* dst, uint64_t& cnt, uint8_t& flags) {
        /* fragRayCast.glsl:113-207 per brick, in double precision */
        double invmv[16], invp[16];
        for (int i = 0; i < 16; ++i)
        {
            invmv[i] = fr.inv_mv[i];
            invp[i] = fr.inv_p[i];
        }
        const double nx = (px + 0.5) * 2.0 / W - 1.0;
        const double ny = (py + 0.5) * 2.0 / H - 1.0;
        double e[4];
        for (int i = 0; i < 4; ++i)
            e[i] = invp[0 * 4 + i] * nx + invp[1 * 4 + i] * ny -
                   invp[2 * 4 + i] + invp[3 * 4 + i];
        const double ep[3] = {e[0] / e[3], e[1] / e[3], e[2] / e[3]};
        double eye[3], d[3];
        for (int i = 0; i < 3; ++i)
        {
            eye[i] = invmv[12 + i];
            const double pw = invmv[i] * ep[0] + invmv[4 + i] * ep[1] +
                              invmv[8 + i] * ep[2] + invmv[12 + i];
            d[i] = pw - eye[i];
        }
        const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int i = 0; i < 3; ++i)
            d[i] /= len;
        const double lenE =
            std::sqrt(ep[0] * ep[0] + ep[1] * ep[1] + ep[2] * ep[2]);
        const double tNP = -double(fr.nearp) / (ep[2] / lenE);
        double gmn[3], gmx[3];
        for (int a = 0; a < 3; ++a)
        {
            gmn[a] = gmin[a];
            gmx[a] = gmax[a];
        }
        double tg, tgf;
        intersect64(eye, d, gmn, gmx, tg, tgf);
        const double stepd = 1.0 / double(view->n_samples);
        /* grid index of the previous composited brick's last sample, and
         * that brick's exit parameter (diagnostics only) */
        int64_t prev_k = INT64_MIN;
        double prev_tf = 0.0;
        for (uint32_t oi = 0; oi < n_nodes; ++oi)
        {
            if (dst[3] > sh.early)
                break;
            const uint32_t n = order[oi];
            float bmin[3], bmax[3];
            world_box(*vol, node_ids[n], bmin, bmax);
            double bmn[3], bmx[3];
            for (int a = 0; a < 3; ++a)
            {
                bmn[a] = bmin[a];
                bmx[a] = bmax[a];
            }
            double tn, tf;
            if (!intersect64(eye, d, bmn, bmx, tn, tf) || tf < tNP)
                continue;
            if (tn < tNP)
                tn = tNP;
            const double res = std::fmod(tn - tg, stepd);
            const double residu = res < 0 ? res + stepd : res;
            if (residu > 0.0)
                tn += stepd - residu;
            if (tn > tf)
                continue;
            for (uint32_t c = 0; c < view->n_clip; ++c)
            {
                const float* cp = view->clip[c];
                double rn = d[0] * cp[0] + d[1] * cp[1] + d[2] * cp[2];
                if (rn == 0.0)
                    rn = 1e-10;
                const double t =
                    -(cp[0] * eye[0] + cp[1] * eye[1] + cp[2] * eye[2] + cp[3]) / rn;
                if (rn > 0.0)
                    tn = std::max(tn, t);
                else
                    tf = std::min(tf, t);
            }
            if (tn > tf)
                continue;
            const double t_entry = tn;
            int64_t k_first = INT64_MIN, k_last = INT64_MIN;
            for (double t = tn; t < tf; t += stepd)
            {
                const int64_t kg = std::llround((t - tg) / stepd);
                if (k_first == INT64_MIN)
                    k_first = kg;
                k_last = kg;
                double sv[3];
                for (int a = 0; a < 3; ++a)
                {
                    const double p = eye[a] + d[a] * t;
                    sv[a] = (p - bmn[a]) / (bmx[a] - bmn[a]) * double(rs.B[a]) +
                            double(rs.O[a]);
                }
                const double val = rs.sample(n, sv, view->filter);
                const double dens = val * sh.mul + sh.add;
                double src[4];
                sh.tf_lookup(dens, src);
                sh.composite(src, dst);
                ++cnt;
                if (dst[3] > sh.early)
                    break;
            }
            if (k_first != INT64_MIN)
            {
                if (prev_k != INT64_MIN)
                {
                    if (k_first == prev_k)
                        flags |= OR_PX_DUPLICATE;
                    else if (k_first < prev_k)
                        flags |= OR_PX_INVERTED;
                    else if (k_first > prev_k + 1 && t_entry_face(prev_tf, t_entry))
                        flags |= OR_PX_GAP;
                }
                prev_k = k_last;
                prev_tf = tf;
            }
        }
    };

    auto worker = [&]() {
        uint64_t cnt = 0;
        for (;;)
        {
            const uint32_t y = next_row.fetch_add(1);
            if (y >= row_end)
                break;
            for (uint32_t x = 0; x < W; ++x)
            {
                double* dst = out + (size_t(y) * W + x) * 4;
                if (!accumulate)
                    dst[0] = dst[1] = dst[2] = dst[3] = 0.0;
                const uint64_t before = cnt;
                uint8_t flags = 0;
                if (base_mode == OR_MODE_SHADER)
                    shader(x, y, dst, cnt, flags);
                else
                    per_ray(x, y, dst, cnt);
                const size_t pi = size_t(y) * W + x;
                if (px_samples)
                    px_samples[pi] = uint32_t(cnt - before);
                if (px_flags)
                    px_flags[pi] = flags;
            }
        }
        total_samples += cnt;
    };
    int nt = n_threads > 0 ? n_threads : int(std::thread::hardware_concurrency());
    if (nt < 1)
        nt = 1;
    std::vector<std::thread> pool;
    for (int i = 1; i < nt; ++i)
        pool.emplace_back(worker);
    worker();
    for (auto& t : pool)
        t.join();
    if (n_samples_out)
        *n_samples_out = total_samples.load();
    return 0;
}

} // extern "C"
