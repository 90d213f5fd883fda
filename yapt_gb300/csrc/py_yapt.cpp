// py_yapt: the reference's Python module (PYBIND11_MODULE(py_yapt),
// Source/Python/srcBindings/BindingsGeneral.cpp:42) rebuilt headless over the C ABI of
// yapt_gpu.h. Class, method and enum names follow the reference bindings
// (PyRenderer.cpp:123-137, PyScene.cpp:83-92, PyMaterial.cpp:332-405, PyMesh.cpp:108-132,
// PyTransform.cpp:93-112, PyCamera.cpp, PyLight.cpp, PyRendererVar.cpp:213-238,
// PyReadback.cpp:143-167, PyGLMTypes.cpp:113-118, PyRendererBasicTypes.cpp).
//
// Headless model: Renderer.init creates one device context; Scene.update(dt) commits the
// scene's changes and renders one frame (one sample per pixel at the next Sobol index) into
// the renderer's accumulation film, as CScene::update -> Renderer::render does
// (Source/Scene/src/CScene.cpp:36-66). Any change of geometry, materials, transforms,
// camera or renderer variables restarts the accumulation. readback() returns the film
// synchronously (state Ready). There is no window: setRenderOutputToSurface raises.
//
// Punctual lights follow LightManager::fillParameters (LightManager.cpp:97-107): position is
// the node's world translation, direction the world forward axis (0, 0, -1) rotated by the
// node's transform, intensity colour x max(0, intensity); lights with zero intensity are
// left out.
//
// Textures: Renderer.createTexture (2D, or a cube map of six square slices; RGBA8_UNORM, RGBA8_SRGB
// or RGBA32_SFLOAT), Texture.upload of mip 0 (any range of a cube map's faces),
// Material.set{Albedo,Normal,ORM,Emissive}Texture(texture, uv scale) and the World.Skycube variable
// (a longitude-latitude map, or a cube map: envType ENVIRONMENT_TYPE_CUBE).
//
// Not built (they raise): other texture kinds, debug render pipelines, orthographic cameras.
#include <pybind11/operators.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <dlfcn.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "yapt_gpu.h"

namespace py = pybind11;

namespace pyyapt
{

// ------------------------------------------------------------------ errors
struct YaptError : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

void check(int rc, const char* what)
{
    if (rc != YG_OK) throw YaptError(std::string(what) + ": " + yg_last_error());
}

// ------------------------------------------------------------------ vectors (PyGLMTypes.cpp)
template <typename T, int N>
struct Vec
{
    std::array<T, N> v{};
};
using vec2 = Vec<float, 2>;
using vec3 = Vec<float, 3>;
using vec4 = Vec<float, 4>;
using ivec2 = Vec<int32_t, 2>;
using ivec3 = Vec<int32_t, 3>;
using ivec4 = Vec<int32_t, 4>;

template <typename T, int N>
void bindVec(py::module_& m, const char* name)
{
    using V = Vec<T, N>;
    py::class_<V> c(m, name);
    c.def(py::init<>());
    c.def(py::init([](T s) {
        V r;
        r.v.fill(s);
        return r;
    }));
    c.def(py::init([](std::array<T, N> a) {
        V r;
        r.v = a;
        return r;
    }));
    c.def("__add__", [](const V& a, const V& b) {
        V r;
        for (int i = 0; i < N; ++i) r.v[i] = a.v[i] + b.v[i];
        return r;
    });
    c.def("__sub__", [](const V& a, const V& b) {
        V r;
        for (int i = 0; i < N; ++i) r.v[i] = a.v[i] - b.v[i];
        return r;
    });
    c.def("__mul__", [](const V& a, const V& b) {
        V r;
        for (int i = 0; i < N; ++i) r.v[i] = a.v[i] * b.v[i];
        return r;
    });
    c.def("__truediv__", [](const V& a, const V& b) {
        V r;
        for (int i = 0; i < N; ++i) r.v[i] = a.v[i] / b.v[i];
        return r;
    });
    c.def("__mul__", [](const V& a, T s) {
        V r;
        for (int i = 0; i < N; ++i) r.v[i] = a.v[i] * s;
        return r;
    });
    c.def("__truediv__", [](const V& a, T s) {
        V r;
        for (int i = 0; i < N; ++i) r.v[i] = a.v[i] / s;
        return r;
    });
    c.def("__getitem__", [](const V& a, size_t i) {
        if (i >= (size_t)N) throw py::index_error("vector index out of range");
        return a.v[i];
    });
    c.def("__setitem__", [](V& a, size_t i, T x) {
        if (i >= (size_t)N) throw py::index_error("vector index out of range");
        a.v[i] = x;
    });
    c.def("__len__", [](const V&) { return N; });
    c.def("__eq__", [](const V& a, const V& b) { return a.v == b.v; });
    c.def("__repr__", [](const V& a) {
        std::string s = "vec( ";
        for (int i = 0; i < N; ++i) s += std::to_string(a.v[i]) + (i + 1 < N ? ", " : " )");
        return s;
    });
}

// ------------------------------------------------------------------ small double matrix helpers
struct M4
{
    double a[4][4]; // row-major, column vectors
};

M4 identity()
{
    M4 m{};
    for (int i = 0; i < 4; ++i) m.a[i][i] = 1.0;
    return m;
}

M4 mul(const M4& x, const M4& y)
{
    M4 r{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
        {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += x.a[i][k] * y.a[k][j];
            r.a[i][j] = s;
        }
    return r;
}

// inverse by the adjugate (cofactors of 2x2 minors)
M4 inverse(const M4& m)
{
    const double* a = &m.a[0][0];
    double s0 = a[0] * a[5] - a[4] * a[1], s1 = a[0] * a[6] - a[4] * a[2], s2 = a[0] * a[7] - a[4] * a[3];
    double s3 = a[1] * a[6] - a[5] * a[2], s4 = a[1] * a[7] - a[5] * a[3], s5 = a[2] * a[7] - a[6] * a[3];
    double c5 = a[10] * a[15] - a[14] * a[11], c4 = a[9] * a[15] - a[13] * a[11], c3 = a[9] * a[14] - a[13] * a[10];
    double c2 = a[8] * a[15] - a[12] * a[11], c1 = a[8] * a[14] - a[12] * a[10], c0 = a[8] * a[13] - a[12] * a[9];
    double det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    if (det == 0.0 || !std::isfinite(det)) throw YaptError("singular transform");
    double id = 1.0 / det;
    M4 r;
    double* b = &r.a[0][0];
    b[0] = (a[5] * c5 - a[6] * c4 + a[7] * c3) * id;
    b[1] = (-a[1] * c5 + a[2] * c4 - a[3] * c3) * id;
    b[2] = (a[13] * s5 - a[14] * s4 + a[15] * s3) * id;
    b[3] = (-a[9] * s5 + a[10] * s4 - a[11] * s3) * id;
    b[4] = (-a[4] * c5 + a[6] * c2 - a[7] * c1) * id;
    b[5] = (a[0] * c5 - a[2] * c2 + a[3] * c1) * id;
    b[6] = (-a[12] * s5 + a[14] * s2 - a[15] * s1) * id;
    b[7] = (a[8] * s5 - a[10] * s2 + a[11] * s1) * id;
    b[8] = (a[4] * c4 - a[5] * c2 + a[7] * c0) * id;
    b[9] = (-a[0] * c4 + a[1] * c2 - a[3] * c0) * id;
    b[10] = (a[12] * s4 - a[13] * s2 + a[15] * s0) * id;
    b[11] = (-a[8] * s4 + a[9] * s2 - a[11] * s0) * id;
    b[12] = (-a[4] * c3 + a[5] * c1 - a[6] * c0) * id;
    b[13] = (a[0] * c3 - a[1] * c1 + a[2] * c0) * id;
    b[14] = (-a[12] * s3 + a[13] * s1 - a[14] * s0) * id;
    b[15] = (a[8] * s3 - a[9] * s1 + a[10] * s0) * id;
    return r;
}

// rotation of the unit quaternion (x, y, z, w)
void quatToMatrix(const vec4& q, double R[3][3])
{
    double x = q.v[0], y = q.v[1], z = q.v[2], w = q.v[3];
    R[0][0] = 1 - 2 * (y * y + z * z);
    R[0][1] = 2 * (x * y - w * z);
    R[0][2] = 2 * (x * z + w * y);
    R[1][0] = 2 * (x * y + w * z);
    R[1][1] = 1 - 2 * (x * x + z * z);
    R[1][2] = 2 * (y * z - w * x);
    R[2][0] = 2 * (x * z - w * y);
    R[2][1] = 2 * (y * z + w * x);
    R[2][2] = 1 - 2 * (x * x + y * y);
}

// quaternion of a rotation matrix: the component of largest magnitude is taken from the
// diagonal and the others from the off-diagonal sums (Shepperd's method)
vec4 matrixToQuat(const double R[3][3])
{
    double t[4] = {R[0][0] + R[1][1] + R[2][2], R[0][0] - R[1][1] - R[2][2], R[1][1] - R[0][0] - R[2][2],
                   R[2][2] - R[0][0] - R[1][1]};
    int k = 0;
    for (int i = 1; i < 4; ++i)
        if (t[i] > t[k]) k = i;
    double big = std::sqrt(t[k] + 1.0) * 0.5, f = 0.25 / big;
    double x, y, z, w;
    switch (k)
    {
    case 0: w = big, x = (R[2][1] - R[1][2]) * f, y = (R[0][2] - R[2][0]) * f, z = (R[1][0] - R[0][1]) * f; break;
    case 1: x = big, w = (R[2][1] - R[1][2]) * f, y = (R[1][0] + R[0][1]) * f, z = (R[0][2] + R[2][0]) * f; break;
    case 2: y = big, w = (R[0][2] - R[2][0]) * f, x = (R[1][0] + R[0][1]) * f, z = (R[2][1] + R[1][2]) * f; break;
    default: z = big, w = (R[1][0] - R[0][1]) * f, x = (R[0][2] + R[2][0]) * f, y = (R[2][1] + R[1][2]) * f; break;
    }
    vec4 q;
    q.v = {(float)x, (float)y, (float)z, (float)w};
    return q;
}

vec4 quatMul(const vec4& a, const vec4& b)
{
    double ax = a.v[0], ay = a.v[1], az = a.v[2], aw = a.v[3];
    double bx = b.v[0], by = b.v[1], bz = b.v[2], bw = b.v[3];
    vec4 r;
    r.v = {(float)(aw * bx + ax * bw + ay * bz - az * by), (float)(aw * by - ax * bz + ay * bw + az * bx),
           (float)(aw * bz + ax * by - ay * bx + az * bw), (float)(aw * bw - ax * bx - ay * by - az * bz)};
    return r;
}

// ------------------------------------------------------------------ Transform (Transform.inl)
struct TransformData
{
    vec3 translation{};
    vec4 orientation{{0.f, 0.f, 0.f, 1.f}};
    vec3 scale{{1.f, 1.f, 1.f}};
    std::shared_ptr<TransformData> parent;

    // object-to-world: parent * T * R * S (Transform::calculateMatrixOS and getMatrixWS)
    M4 world() const
    {
        double R[3][3];
        quatToMatrix(orientation, R);
        M4 m = identity();
        for (int i = 0; i < 3; ++i)
        {
            for (int j = 0; j < 3; ++j) m.a[i][j] = R[i][j] * (double)scale.v[j];
            m.a[i][3] = translation.v[i];
        }
        return parent ? mul(parent->world(), m) : m;
    }
};

struct Transform
{
    std::shared_ptr<TransformData> d;

    void setTranslation(const vec3& v) { d->translation = v; }
    void addTranslation(const vec3& v)
    {
        for (int i = 0; i < 3; ++i) d->translation.v[i] += v.v[i];
    }
    vec3 getTranslation() const { return d->translation; }
    void setScale(const vec3& v) { d->scale = v; }
    // the reference's addScale assigns the scale (Transform.inl: addScale)
    void addScale(const vec3& v) { d->scale = v; }
    vec3 getScale() const { return d->scale; }
    void setOrientation(const vec4& q) { d->orientation = q; }
    void addOrientation(const vec4& q) { d->orientation = quatMul(d->orientation, q); }
    vec4 getOrientation() const { return d->orientation; }
    // camera-style look-at: the object looks down its local -z from `eye` (Transform::lookAt)
    void lookAt(const vec3& eye, const vec3& at, const vec3& up)
    {
        double f[3], s[3], u[3];
        double n = 0;
        for (int i = 0; i < 3; ++i) n += (double(at.v[i]) - eye.v[i]) * (double(at.v[i]) - eye.v[i]);
        n = std::sqrt(n);
        if (!(n > 0)) throw YaptError("lookAt: eye and target coincide");
        for (int i = 0; i < 3; ++i) f[i] = (double(at.v[i]) - eye.v[i]) / n;
        s[0] = f[1] * up.v[2] - f[2] * up.v[1];
        s[1] = f[2] * up.v[0] - f[0] * up.v[2];
        s[2] = f[0] * up.v[1] - f[1] * up.v[0];
        double sn = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
        if (!(sn > 0)) throw YaptError("lookAt: up is parallel to the view direction");
        for (double& c : s) c /= sn;
        u[0] = s[1] * f[2] - s[2] * f[1];
        u[1] = s[2] * f[0] - s[0] * f[2];
        u[2] = s[0] * f[1] - s[1] * f[0];
        double R[3][3];
        for (int i = 0; i < 3; ++i)
        {
            R[i][0] = s[i];
            R[i][1] = u[i];
            R[i][2] = -f[i];
        }
        d->orientation = matrixToQuat(R);
        d->translation = eye;
        d->scale.v = {1.f, 1.f, 1.f};
    }
    void setParent(py::object other)
    {
        if (other.is_none())
        {
            d->parent.reset();
            return;
        }
        Transform t = other.cast<Transform>();
        for (auto p = t.d; p; p = p->parent)
            if (p == d) throw YaptError("setParent: the parent chain would contain a cycle");
        d->parent = t.d;
    }
    uintptr_t getId() const { return reinterpret_cast<uintptr_t>(d.get()); }
    uintptr_t getParentId() const { return reinterpret_cast<uintptr_t>(d->parent.get()); }
    vec3 axis(double x, double y, double z) const
    {
        M4 w = d->world();
        vec3 r;
        for (int i = 0; i < 3; ++i) r.v[i] = (float)(w.a[i][0] * x + w.a[i][1] * y + w.a[i][2] * z);
        return r;
    }
    std::vector<std::vector<double>> getMatrixWS() const
    {
        M4 w = d->world();
        std::vector<std::vector<double>> r(4, std::vector<double>(4));
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) r[i][j] = w.a[i][j];
        return r;
    }
};

// ------------------------------------------------------------------ enums (GfxBasicTypes)
enum class AttributeSemanticName : int
{
    UNKNOWN = 0,
    POSITION,
    TEXCOORD,
    NORMAL,
    TANGENT,
    COLOR
};
enum class ResourceDimension : int
{
    BUFFER = 0,
    TEXTURE_1D,
    TEXTURE_1D_ARRAY,
    TEXTURE_2D,
    TEXTURE_2D_ARRAY,
    TEXTURE_3D,
    TEXTURE_CUBEMAP,
    TEXTURE_CUBEMAP_ARRAY,
    UNDEFINED
};
// the formats mesh data and readbacks use, under the reference's names
#define YG_FORMATS(X)                                                                                                   \
    X(UNKNOWN, 0) X(R8_UNORM, 1) X(R16_UINT, 2) X(R16_SFLOAT, 2) X(R32_UINT, 4) X(R32_SINT, 4) X(R32_SFLOAT, 4)             \
    X(RG16_SFLOAT, 4) X(RG32_UINT, 8) X(RG32_SINT, 8) X(RG32_SFLOAT, 8) X(RGB32_UINT, 12) X(RGB32_SINT, 12)               \
    X(RGB32_SFLOAT, 12) X(RGBA8_UNORM, 4) X(RGBA8_UINT, 4) X(RGBA8_SRGB, 4) X(RGBA16_UNORM, 8) X(RGBA16_SFLOAT, 8)         \
    X(RGBA32_UINT, 16) X(RGBA32_SINT, 16) X(RGBA32_SFLOAT, 16)
enum class ResourceFormat : int
{
#define YG_ENUM(n, s) n,
    YG_FORMATS(YG_ENUM)
#undef YG_ENUM
};
uint32_t formatSize(ResourceFormat f)
{
    switch (f)
    {
#define YG_SIZE(n, s)                                                                                                   \
    case ResourceFormat::n: return s;
        YG_FORMATS(YG_SIZE)
#undef YG_SIZE
    }
    return 0;
}
enum ResourceUsageBits : uint32_t
{
    RESOURCE_USAGE_UNKNOWN = 0,
    RESOURCE_USAGE_COPY_DESTINATION = 1u << 0,
    RESOURCE_USAGE_COPY_SOURCE = 1u << 1,
    RESOURCE_USAGE_UNIFORM_BUFFER = 1u << 2,
    RESOURCE_USAGE_STORAGE_BUFFER = 1u << 3,
    RESOURCE_USAGE_VERTEX_BUFFER = 1u << 4,
    RESOURCE_USAGE_INDEX_BUFFER = 1u << 5,
    RESOURCE_USAGE_ACCELERATION_STRUCTURE_BUILD_INPUT = 1u << 6,
    RESOURCE_USAGE_SAMPLED_TEXTURE = 1u << 7,
    RESOURCE_USAGE_STORAGE_TEXTURE = 1u << 8
};
enum class LightType : int
{
    POINT = 0,
    SPOT,
    DIRECTIONAL
};
enum class ProjectionType : int
{
    PERSPECTIVE = 0,
    ORTHOGRAPHIC
};
enum class ReadbackTarget : int
{
    FinalColor = 0, // RGBA8_UNORM, sRGB-encoded exposure x linear sRGB of the film, clamped
    FilmXYZ,        // RGBA32_SFLOAT: mean XYZ and the sample count
    FilmRGB,        // RGBA32_SFLOAT: mean linear sRGB and the sample count
    Features        // RGBA32_SFLOAT, 2 slices: albedo rgb + depth, normal xyz + 0
};
enum class ReadbackState : int
{
    Created = 0,
    Pending,
    Ready,
    Failed,
    Freed
};
enum class RendererVariableType : int
{
    FLOAT = 0,
    INT,
    TEXTURE,
    BUFFER,
    OPTIONS
};
enum class MaterialPreset : int
{
    BLANK = 0,
    METAL_GOLD,
    METAL_SILVER,
    METAL_COPPER,
    METAL_BRASS,
    METAL_ALUMINIUM,
    GLASS,
    PLASTIC
};

// ------------------------------------------------------------------ Buffer / Mesh
struct BufferData
{
    std::string name;
    uint32_t usage = 0;
    std::vector<uint8_t> bytes;
    uint64_t version = 0;
};

struct Buffer
{
    std::shared_ptr<BufferData> d;
    // PyBuffer::upload(offsetInBytes, sizeInBytes, data, dataPtrOffset): copies from a host address
    void upload(size_t offset, size_t size, uintptr_t data, size_t dataOffset)
    {
        if (offset + size > d->bytes.size()) throw YaptError("Buffer.upload: range outside the buffer");
        if (size && !data) throw YaptError("Buffer.upload: null data");
        std::memcpy(d->bytes.data() + offset, reinterpret_cast<const uint8_t*>(data) + dataOffset, size);
        ++d->version;
    }
    std::string getName() const { return d->name; }
};

struct MeshAttribute
{
    ResourceFormat format = ResourceFormat::UNKNOWN;
    AttributeSemanticName semanticName = AttributeSemanticName::UNKNOWN;
    uint32_t semanticIndex = 0;
    uint32_t offset = 0xFFFFFFFFu; // Attribute::INFER_OFFSET_FROM_LAYOUT
};

struct VertexBufferLayout
{
    std::vector<MeshAttribute> attributes;
    uint32_t vertexStrideInBytes = 0xFFFFFFFFu; // VERTEX_STRIDE_TIGHTLY_PACKED
    static constexpr uint32_t STRIDE_TIGHTLY_PACKED = 0xFFFFFFFFu;
};

struct Submesh
{
    size_t indexOffset = 0, indexCount = 0, vertexOffset = 0;
    bool set = false;
};

struct MeshData
{
    std::string name;
    std::vector<VertexBufferLayout> layouts;
    size_t vertexCount = 0;
    bool use16 = false;
    std::vector<std::shared_ptr<BufferData>> vbuf;
    std::vector<size_t> vbufOffset;
    std::shared_ptr<BufferData> ibuf;
    size_t ibufOffset = 0;
    std::vector<Submesh> submeshes;
    uint64_t version = 0;

    uint64_t contentVersion() const
    {
        uint64_t v = version;
        for (auto& b : vbuf) v = v * 1000003u + (b ? b->version + 1 : 0);
        return v * 1000003u + (ibuf ? ibuf->version + 1 : 0);
    }
};

// vertex streams of a mesh decoded from its buffers and layouts (MeshProxy.cpp:15-70 rules:
// offsets inferred as running sums, stride the packed size unless given)
struct DecodedMesh
{
    std::vector<float> positions, normals, tangents, uvs;
    std::vector<uint32_t> indices;   // absolute vertex indices (submesh vertex offsets applied)
    std::vector<uint32_t> submeshes; // (first index, index count) pairs
    bool hasTangents = false, hasUvs = false;
};

DecodedMesh decodeMesh(const MeshData& m)
{
    struct Stream
    {
        int buffer = -1;
        uint32_t offset = 0, stride = 0;
        ResourceFormat format = ResourceFormat::UNKNOWN;
    } pos, nrm, tan, uv;
    for (size_t b = 0; b < m.layouts.size(); ++b)
    {
        const VertexBufferLayout& L = m.layouts[b];
        uint32_t total = 0;
        std::vector<std::pair<uint32_t, const MeshAttribute*>> offs;
        for (const MeshAttribute& a : L.attributes)
        {
            uint32_t off = a.offset == 0xFFFFFFFFu ? total : a.offset;
            offs.push_back({off, &a});
            total = off + formatSize(a.format);
        }
        uint32_t stride = L.vertexStrideInBytes == VertexBufferLayout::STRIDE_TIGHTLY_PACKED ? total : L.vertexStrideInBytes;
        for (auto& [off, a] : offs)
        {
            if (a->semanticIndex != 0) continue;
            Stream s{(int)b, off, stride, a->format};
            if (a->semanticName == AttributeSemanticName::POSITION) pos = s;
            else if (a->semanticName == AttributeSemanticName::NORMAL) nrm = s;
            else if (a->semanticName == AttributeSemanticName::TANGENT) tan = s;
            else if (a->semanticName == AttributeSemanticName::TEXCOORD) uv = s;
        }
    }
    if (pos.buffer < 0) throw YaptError("mesh '" + m.name + "': no POSITION attribute");
    if (nrm.buffer < 0) throw YaptError("mesh '" + m.name + "': no NORMAL attribute");
    auto fetch = [&](const Stream& s, int comps, std::vector<float>& out) {
        if (s.format != ResourceFormat::RGB32_SFLOAT && s.format != ResourceFormat::RGBA32_SFLOAT &&
            s.format != ResourceFormat::RG32_SFLOAT)
            throw YaptError("mesh '" + m.name + "': vertex attributes must be 32-bit float vectors");
        int have = (int)formatSize(s.format) / 4;
        if (have < comps) throw YaptError("mesh '" + m.name + "': attribute has too few components");
        const auto& buf = m.vbuf.at(s.buffer);
        if (!buf) throw YaptError("mesh '" + m.name + "': vertex buffer not set");
        size_t base = m.vbufOffset[s.buffer];
        out.resize(m.vertexCount * comps);
        for (size_t v = 0; v < m.vertexCount; ++v)
        {
            size_t at = base + v * s.stride + s.offset;
            if (at + 4 * comps > buf->bytes.size()) throw YaptError("mesh '" + m.name + "': vertex buffer too small");
            std::memcpy(&out[v * comps], buf->bytes.data() + at, 4 * comps);
        }
    };
    DecodedMesh d;
    fetch(pos, 3, d.positions);
    fetch(nrm, 3, d.normals);
    if (tan.buffer >= 0)
    {
        fetch(tan, 4, d.tangents);
        d.hasTangents = true;
    }
    if (uv.buffer >= 0)
    {
        fetch(uv, 2, d.uvs);
        d.hasUvs = true;
    }
    if (!m.ibuf) throw YaptError("mesh '" + m.name + "': index buffer not set");
    const size_t isz = m.use16 ? 2 : 4;
    for (size_t s = 0; s < m.submeshes.size(); ++s)
    {
        const Submesh& sm = m.submeshes[s];
        if (!sm.set) throw YaptError("mesh '" + m.name + "': submesh " + std::to_string(s) + " not set");
        d.submeshes.push_back((uint32_t)d.indices.size());
        d.submeshes.push_back((uint32_t)sm.indexCount);
        for (size_t i = 0; i < sm.indexCount; ++i)
        {
            size_t at = m.ibufOffset + (sm.indexOffset + i) * isz;
            if (at + isz > m.ibuf->bytes.size()) throw YaptError("mesh '" + m.name + "': index buffer too small");
            uint32_t v = 0;
            std::memcpy(&v, m.ibuf->bytes.data() + at, isz);
            d.indices.push_back((uint32_t)(v + sm.vertexOffset));
        }
    }
    return d;
}

struct Mesh
{
    std::shared_ptr<MeshData> d;
    std::string getName() const { return d->name; }
    void setVertexBuffer(size_t index, const Buffer& b, size_t offset)
    {
        if (index >= d->vbuf.size()) throw YaptError("Mesh.setVertexBuffer: no layout with this index");
        d->vbuf[index] = b.d;
        d->vbufOffset[index] = offset;
        ++d->version;
    }
    void setIndexBuffer(const Buffer& b, size_t offset)
    {
        d->ibuf = b.d;
        d->ibufOffset = offset;
        ++d->version;
    }
    void setSubmesh(size_t index, size_t indexOffset, size_t indexCount, size_t vertexOffset, const vec3&, const vec3&)
    {
        if (index >= d->submeshes.size()) throw YaptError("Mesh.setSubmesh: submesh index out of range");
        if (indexCount % 3) throw YaptError("Mesh.setSubmesh: index count must be a multiple of 3");
        d->submeshes[index] = Submesh{indexOffset, indexCount, vertexOffset, true};
        ++d->version;
    }
    size_t getSubmeshCount() const { return d->submeshes.size(); }
    // the vertex streams and indices the renderer uploads for this mesh
    py::dict decoded() const
    {
        DecodedMesh m = decodeMesh(*d);
        py::dict r;
        r["positions"] = m.positions;
        r["normals"] = m.normals;
        r["tangents"] = m.tangents;
        r["uvs"] = m.uvs;
        r["indices"] = m.indices;
        r["submeshes"] = m.submeshes;
        return r;
    }
};

// PyMesh::calculateBoundsFromVertexBuffer: bounds of the indexed vertices of a submesh
py::tuple calculateBounds(uintptr_t vertexData, uintptr_t indexData, size_t indexOffset, size_t indexCount,
                          size_t vertexOffset, size_t vertexStride, bool use16)
{
    vec3 lo, hi;
    lo.v.fill(INFINITY);
    hi.v.fill(-INFINITY);
    const char* vp = reinterpret_cast<const char*>(vertexData);
    const char* ip = reinterpret_cast<const char*>(indexData);
    size_t isz = use16 ? 2 : 4;
    for (size_t i = 0; i < indexCount; ++i)
    {
        uint32_t idx = 0;
        std::memcpy(&idx, ip + (i + indexOffset) * isz, isz);
        float p[3];
        std::memcpy(p, vp + (idx + vertexOffset) * vertexStride, sizeof(p));
        for (int k = 0; k < 3; ++k)
        {
            lo.v[k] = std::min(lo.v[k], p[k]);
            hi.v[k] = std::max(hi.v[k], p[k]);
        }
    }
    return py::make_tuple(lo, hi);
}

// ------------------------------------------------------------------ Material (MaterialProxy)
constexpr float kSpecLmin = 380.f, kSpecLmax = 780.f;
constexpr int kSpecPoints = 81; // 5 nm grid

// Texture (PyTexture.cpp): a 2D texture held on the host until a scene update uploads the
// textures its materials and the skybox use (yg_upload_texture)
struct TextureData
{
    std::string name;
    uint32_t format = YG_TEXTURE_RGBA8_UNORM; // YG_TEXTURE_*
    uint32_t width = 0, height = 0;
    uint32_t layers = 1;         // 6 for a cube map (faces +X, -X, +Y, -Y, +Z, -Z)
    std::vector<uint8_t> texels; // mip 0, rows packed, layer after layer
    uint64_t version = 0;
};

struct MaterialData
{
    std::string name;
    yg_material m{};
    std::shared_ptr<TextureData> tex[4]; // albedo, normal, ORM, emissive
    bool twoSided = false, dispersion = false, alphaBlend = false;
    std::vector<float> albedoSpec, specularSpec, emissionSpec; // empty: RGB
    uint64_t version = 0;
};

// MaterialParameters() defaults (MaterialInternal.h:41-77)
void setDefaults(MaterialData& d)
{
    yg_material& m = d.m;
    std::memset(&m, 0, sizeof(m));
    m.albedo[0] = m.albedo[1] = m.albedo[2] = 1.f;
    m.specular[0] = m.specular[1] = m.specular[2] = 1.f;
    m.metalness = 1.f;
    m.dielectric_ior = 1.5f;
    m.roughness = 0.1f;
    m.specular_amount = 1.f;
    m.clear_coat_ior = 1.5f;
    m.clear_coat_roughness = 0.1f;
    m.sheen_tint[0] = m.sheen_tint[1] = m.sheen_tint[2] = 1.f;
    m.sheen_roughness = 0.5f;
    m.cauchy[0] = 1.5046f;
    m.cauchy[1] = 0.00420f;
    m.subsurface_radius[0] = 1.f;
    m.subsurface_radius[1] = 0.2f;
    m.subsurface_radius[2] = 0.1f;
    m.subsurface_radius_scale = 1.f;
    m.albedo_spectrum = m.specular_spectrum = m.emission_spectrum = -1;
    d.twoSided = d.dispersion = d.alphaBlend = false;
    d.albedoSpec.clear();
    d.specularSpec.clear();
    d.emissionSpec.clear();
}

// piecewise-linear resampling onto the 5 nm grid, ends held (numpy.interp)
std::vector<float> resample(const std::vector<double>& lam, const std::vector<double>& val)
{
    if (lam.size() != val.size()) throw YaptError("spectrum: wavelengths and values differ in length");
    if (lam.empty()) return {};
    for (size_t i = 1; i < lam.size(); ++i)
        if (!(lam[i] > lam[i - 1])) throw YaptError("spectrum: wavelengths must increase");
    std::vector<float> out(kSpecPoints);
    for (int i = 0; i < kSpecPoints; ++i)
    {
        double x = kSpecLmin + 5.0 * i;
        double y;
        if (x <= lam.front()) y = val.front();
        else if (x >= lam.back()) y = val.back();
        else
        {
            size_t j = std::upper_bound(lam.begin(), lam.end(), x) - lam.begin() - 1;
            double slope = (val[j + 1] - val[j]) / (lam[j + 1] - lam[j]);
            y = slope * (x - lam[j]) + val[j];
        }
        out[i] = (float)y;
    }
    return out;
}

struct Material
{
    std::shared_ptr<MaterialData> d;
    void touch() { ++d->version; }
    std::string getName() const { return d->name; }

    void setFromMaterialPreset(MaterialPreset p)
    {
        // MaterialProxy::setFromMaterialPreset (MaterialProxy.cpp:15-55): the ten-argument
        // MaterialParameters constructor, colours given in sRGB and raised to 2.2
        auto g = [](double c) { return (float)std::pow(c, 2.2); };
        auto set10 = [&](std::array<double, 3> alb, float transp, std::array<double, 3> spec, float metal, bool gamma) {
            setDefaults(*d);
            for (int i = 0; i < 3; ++i)
            {
                d->m.albedo[i] = gamma ? g(alb[i]) : (float)alb[i];
                d->m.specular[i] = gamma ? g(spec[i]) : (float)spec[i];
            }
            d->m.transparency = transp;
            d->m.metalness = metal;
            d->m.dielectric_ior = 1.5f;
            d->m.roughness = 0.f;
            d->m.anisotropy = 0.f;
            d->m.anisotropy_rotation = 0.f;
        };
        switch (p)
        {
        case MaterialPreset::BLANK: setDefaults(*d); break;
        case MaterialPreset::METAL_GOLD: set10({0.9451, 0.7294, 0.37255}, 0.f, {1.0, 0.97255, 0.73333}, 1.f, true); break;
        case MaterialPreset::METAL_SILVER: set10({0.9607, 0.9490, 0.9176}, 0.f, {1.0, 1.0, 1.0}, 1.f, true); break;
        case MaterialPreset::METAL_ALUMINIUM: set10({0.9137, 0.9137, 0.9137}, 0.f, {0.9686, 0.98039, 0.9882}, 1.f, true); break;
        case MaterialPreset::METAL_BRASS: set10({0.903, 0.744, 0.473}, 0.f, {0.975, 0.958, 0.918}, 1.f, true); break;
        case MaterialPreset::METAL_COPPER: set10({0.92549, 0.68627, 0.50196}, 0.f, {0.9960, 0.945098, 0.8196}, 1.f, true); break;
        case MaterialPreset::GLASS: set10({1, 1, 1}, 1.f, {1, 1, 1}, 0.f, false); break;
        case MaterialPreset::PLASTIC: set10({1, 1, 1}, 0.f, {1, 1, 1}, 0.f, false); break;
        }
        touch();
    }

#define YG_SCALAR(Name, field)                                                                                          \
    void set##Name(float v)                                                                                             \
    {                                                                                                                   \
        d->m.field = v;                                                                                                 \
        touch();                                                                                                        \
    }                                                                                                                   \
    float get##Name() const { return d->m.field; }
#define YG_VEC3(Name, field)                                                                                            \
    void set##Name(const vec3& v)                                                                                       \
    {                                                                                                                   \
        for (int i = 0; i < 3; ++i) d->m.field[i] = v.v[i];                                                             \
        touch();                                                                                                        \
    }                                                                                                                   \
    vec3 get##Name() const                                                                                              \
    {                                                                                                                   \
        vec3 r;                                                                                                         \
        for (int i = 0; i < 3; ++i) r.v[i] = d->m.field[i];                                                             \
        return r;                                                                                                       \
    }
    YG_SCALAR(Transparency, transparency)
    YG_SCALAR(Metalness, metalness)
    YG_VEC3(Albedo, albedo)
    YG_VEC3(SpecularTint, specular)
    YG_VEC3(Absorption, absorption)
    YG_VEC3(Emission, emissive)
    YG_SCALAR(EmissionFocus, emission_focus)
    YG_SCALAR(DielectricIOR, dielectric_ior)
    YG_SCALAR(Roughness, roughness)
    YG_SCALAR(Anisotropy, anisotropy)
    YG_SCALAR(AnisotropyRotation, anisotropy_rotation)
    YG_SCALAR(SpecularAmount, specular_amount)
    YG_SCALAR(ClearCoatAmount, clear_coat_amount)
    YG_SCALAR(ClearCoatRoughness, clear_coat_roughness)
    YG_SCALAR(ClearCoatIOR, clear_coat_ior)
    YG_SCALAR(SheenRoughness, sheen_roughness)
    YG_VEC3(SheenTint, sheen_tint)
    YG_SCALAR(SheenAmount, sheen_amount)
    YG_SCALAR(AlphaCutoff, alpha_cutoff)
    YG_SCALAR(ThinFilmThicknessNM, thin_film_thickness_nm)
    YG_SCALAR(SubsurfaceAmount, subsurface_amount)
    YG_VEC3(SubsurfaceRadius, subsurface_radius)
    YG_SCALAR(SubsurfaceRadiusScale, subsurface_radius_scale)
#undef YG_SCALAR
#undef YG_VEC3
    void setTwoSided(bool b)
    {
        d->twoSided = b;
        touch();
    }
    bool getTwoSided() const { return d->twoSided; }
    void setAlphaBlend(bool b)
    {
        d->alphaBlend = b;
        touch();
    }
    bool getAlphaBlend() const { return d->alphaBlend; }
    void setEnableDispersion(bool b)
    {
        d->dispersion = b;
        touch();
    }
    bool getEnableDispersion() const { return d->dispersion; }
    void setCauchysCoefficients(const vec2& c)
    {
        d->m.cauchy[0] = c.v[0];
        d->m.cauchy[1] = c.v[1];
        touch();
    }
    vec2 getCauchysCoefficients() const
    {
        vec2 r;
        r.v = {d->m.cauchy[0], d->m.cauchy[1]};
        return r;
    }
    // PyMaterial::set*Texture (PyMaterial.cpp:299-326): the texture and its uv scale
    void setSlot(int k, const std::shared_ptr<TextureData>& t, const vec2& scale)
    {
        if (t && t->layers != 1) throw YaptError("material '" + d->name + "': a material texture is 2D, not a cube map");
        d->tex[k] = t;
        float* s = k == 0 ? d->m.albedo_uv_scale : k == 1 ? d->m.normal_uv_scale : k == 2 ? d->m.orm_uv_scale : d->m.emissive_uv_scale;
        s[0] = scale.v[0];
        s[1] = scale.v[1];
        touch();
    }

    // spectral extension: tabulated curves instead of the RGB -> spectrum conversion
    void setAlbedoSpectrum(const std::vector<double>& lam, const std::vector<double>& val)
    {
        d->albedoSpec = resample(lam, val);
        touch();
    }
    void setSpecularSpectrum(const std::vector<double>& lam, const std::vector<double>& val)
    {
        d->specularSpec = resample(lam, val);
        touch();
    }
    void setEmissionSpectrum(const std::vector<double>& lam, const std::vector<double>& val)
    {
        d->emissionSpec = resample(lam, val);
        touch();
    }
    // Planck's law on the 5 nm grid, normalised to a peak of 1 over 380..780 nm
    void setEmissionBlackbody(double T)
    {
        if (!(T > 0)) throw YaptError("setEmissionBlackbody: temperature must be positive");
        const double h = 6.62607015e-34, c = 2.99792458e8, k = 1.380649e-23;
        std::vector<double> b(kSpecPoints);
        double mx = 0;
        for (int i = 0; i < kSpecPoints; ++i)
        {
            double lam = (kSpecLmin + 5.0 * i) * 1e-9;
            b[i] = (2 * h * c * c) / (lam * lam * lam * lam * lam) / std::expm1(h * c / (lam * k * T));
            mx = std::max(mx, b[i]);
        }
        d->emissionSpec.resize(kSpecPoints);
        for (int i = 0; i < kSpecPoints; ++i) d->emissionSpec[i] = (float)(b[i] / mx);
        touch();
    }
    std::vector<float> getAlbedoSpectrum() const { return d->albedoSpec; }
    std::vector<float> getEmissionSpectrum() const { return d->emissionSpec; }
};

// ------------------------------------------------------------------ Renderer variables
struct VarData
{
    std::string name;
    RendererVariableType type = RendererVariableType::FLOAT;
    int comps = 1;
    std::array<double, 4> val{}, lo{}, hi{};
    std::vector<std::string> options;
    int selected = 0;
    std::shared_ptr<TextureData> texture; // TEXTURE variables
};

struct Texture
{
    std::shared_ptr<TextureData> d;
    // PyTexture::upload: mip 0 of slices [arrayOffset, arrayOffset + arrayCount) (one for a 2D
    // texture, up to six faces of a cube map); rows rowPitchInBytes apart in host memory at
    // data + dataPtrOffset (a numpy array's ctypes.data, as the reference scripts pass it), one
    // slice after the other
    void upload(uint32_t mipOffset, uint32_t arrayOffset, uint32_t mipCount, uint32_t arrayCount, size_t rowPitch,
                uintptr_t data, size_t offset)
    {
        if (mipOffset != 0 || mipCount < 1) throw YaptError("texture '" + d->name + "': only mip 0 is used");
        const uint32_t n = std::max<uint32_t>(arrayCount, 1);
        if (arrayOffset >= d->layers || n > d->layers - arrayOffset)
            throw YaptError("texture '" + d->name + "': slices outside the texture");
        const size_t texel = d->format == YG_TEXTURE_RGBA32_FLOAT ? 16 : 4, row = texel * d->width;
        if (rowPitch < row) throw YaptError("texture '" + d->name + "': row pitch smaller than a row");
        if (!data) throw YaptError("texture '" + d->name + "': null data");
        const uint8_t* src = reinterpret_cast<const uint8_t*>(data) + offset;
        d->texels.resize(row * d->height * d->layers);
        for (uint32_t l = 0; l < n; ++l)
            for (uint32_t y = 0; y < d->height; ++y)
                std::memcpy(d->texels.data() + ((size_t)(arrayOffset + l) * d->height + y) * row,
                            src + ((size_t)l * d->height + y) * rowPitch, row);
        ++d->version;
    }
    std::string getName() const { return d->name; }
};

struct RendererVariable
{
    std::shared_ptr<VarData> d;
    std::shared_ptr<uint64_t> serial; // renderer-wide change counter

    void setFromFloatArray(const std::vector<double>& v)
    {
        if (d->type != RendererVariableType::FLOAT) throw YaptError(d->name + ": not a FLOAT variable");
        if ((int)v.size() != d->comps) throw YaptError(d->name + ": expected " + std::to_string(d->comps) + " values");
        for (int i = 0; i < d->comps; ++i) d->val[i] = std::clamp((double)(float)v[i], d->lo[i], d->hi[i]);
        ++*serial;
    }
    void setFromIntArray(const std::vector<int64_t>& v)
    {
        if (d->type != RendererVariableType::INT) throw YaptError(d->name + ": not an INT variable");
        if ((int)v.size() != d->comps) throw YaptError(d->name + ": expected " + std::to_string(d->comps) + " values");
        for (int i = 0; i < d->comps; ++i) d->val[i] = std::clamp((double)v[i], d->lo[i], d->hi[i]);
        ++*serial;
    }
    void setTexture(const Texture& t)
    {
        if (d->type != RendererVariableType::TEXTURE) throw YaptError(d->name + ": not a TEXTURE variable");
        d->texture = t.d;
        ++*serial;
    }
    py::object getTexture() const
    {
        if (d->type != RendererVariableType::TEXTURE) throw YaptError(d->name + ": not a TEXTURE variable");
        if (!d->texture) return py::none();
        return py::cast(Texture{d->texture});
    }
    std::vector<double> getAsFloatArray() const
    {
        if (d->type != RendererVariableType::FLOAT) throw YaptError(d->name + ": not a FLOAT variable");
        return std::vector<double>(d->val.begin(), d->val.begin() + d->comps);
    }
    std::vector<int64_t> getAsIntArray() const
    {
        if (d->type != RendererVariableType::INT) throw YaptError(d->name + ": not an INT variable");
        std::vector<int64_t> r;
        for (int i = 0; i < d->comps; ++i) r.push_back((int64_t)d->val[i]);
        return r;
    }
    py::tuple getLimitsFloat() const
    {
        return py::make_tuple(std::vector<double>(d->lo.begin(), d->lo.begin() + d->comps),
                              std::vector<double>(d->hi.begin(), d->hi.begin() + d->comps));
    }
    py::tuple getLimitsInt() const
    {
        std::vector<int64_t> lo, hi;
        for (int i = 0; i < d->comps; ++i)
        {
            lo.push_back((int64_t)d->lo[i]);
            hi.push_back((int64_t)d->hi[i]);
        }
        return py::make_tuple(lo, hi);
    }
    int getComponentCount() const { return d->comps; }
    std::vector<std::string> getOptions() const { return d->options; }
    int getSelectedOption() const { return d->selected; }
    void setSelectedOption(int i)
    {
        if (d->type != RendererVariableType::OPTIONS) throw YaptError(d->name + ": not an OPTIONS variable");
        if (i < 0 || i >= (int)d->options.size()) throw YaptError(d->name + ": option index out of range");
        d->selected = i;
        ++*serial;
    }
    RendererVariableType getType() const { return d->type; }
};

// ------------------------------------------------------------------ Readback
struct ReadbackData
{
    size_t width = 0, height = 0, slices = 1;
    ResourceFormat format = ResourceFormat::UNKNOWN;
    std::vector<uint8_t> bytes;
    size_t texel() const { return formatSize(format); }
};

struct ReadbackObject
{
    ReadbackState state = ReadbackState::Created;
    std::shared_ptr<ReadbackData> data;
    ReadbackState getState() const { return state; }
    bool isReady() const { return state == ReadbackState::Ready; }
    void release()
    {
        data.reset();
        state = ReadbackState::Freed;
    }
    std::shared_ptr<ReadbackData> getData() const { return state == ReadbackState::Ready ? data : nullptr; }
};

// ------------------------------------------------------------------ renderer state
struct RendererCacheTag
{
}; // RendererCache: shader/LUT cache of the DX12 renderer; nothing to cache here

std::string packageDataDir()
{
    Dl_info info{};
    if (!dladdr(reinterpret_cast<void*>(&packageDataDir), &info) || !info.dli_fname)
        throw YaptError("cannot locate the module's folder");
    std::string p = info.dli_fname;
    return p.substr(0, p.find_last_of('/')) + "/data";
}

struct RendererState
{
    yg_context* ctx = nullptr;
    std::vector<std::shared_ptr<VarData>> vars;
    std::shared_ptr<uint64_t> serial = std::make_shared<uint64_t>(0);
    // accumulation
    std::vector<uint8_t> lastScene;  // instances, materials, spectra
    std::vector<uint64_t> lastMeshes; // (mesh identity, content version) of the uploaded meshes
    std::vector<uint8_t> lastCamera;
    std::vector<uint8_t> lastLights;
    std::vector<uint64_t> lastTextures; // (pointer, version) of the uploaded textures
    std::vector<uint8_t> lastParams;
    float lastDeltaTime = 0.f;  // Scene.update's deltaTime, the tonemap's eye adaptation step
    bool tonemapStarted = false;
    std::vector<yg_instance> instances; // the records of the last commit
    std::vector<yg_material> materials;
    std::vector<float> spectra;
    yg_camera camera{};
    uint32_t frames = 0;
    uint32_t filmW = 0, filmH = 0;
    bool featuresOn = false;

    ~RendererState()
    {
        if (ctx) yg_destroy(ctx);
    }
    VarData* var(const std::string& n) const
    {
        for (auto& v : vars)
            if (v->name == n) return v.get();
        return nullptr;
    }
    void addFloat(const std::string& n, std::vector<double> def, double lo, double hi)
    {
        auto v = std::make_shared<VarData>();
        v->name = n;
        v->type = RendererVariableType::FLOAT;
        v->comps = (int)def.size();
        for (int i = 0; i < v->comps; ++i) v->val[i] = def[i], v->lo[i] = lo, v->hi[i] = hi;
        vars.push_back(v);
    }
    void addInt(const std::string& n, std::vector<double> def, double lo, double hi)
    {
        addFloat(n, def, lo, hi);
        vars.back()->type = RendererVariableType::INT;
    }
    void addTexture(const std::string& n)
    {
        auto v = std::make_shared<VarData>();
        v->name = n;
        v->type = RendererVariableType::TEXTURE;
        vars.push_back(v);
    }
    void addOptions(const std::string& n, int sel, std::vector<std::string> opts)
    {
        auto v = std::make_shared<VarData>();
        v->name = n;
        v->type = RendererVariableType::OPTIONS;
        v->options = std::move(opts);
        v->selected = sel;
        vars.push_back(v);
    }
};

// renderer variables: the reference's names and defaults (RendererVarsList.h, CRenderer.h:17-47)
// that this renderer honours, and the extensions MaxDepth, Seed, Regularize, spectral range,
// BDPT light-path shape and first-hit features
void registerVariables(RendererState& R)
{
    R.addInt("Generic.RenderResolution", {1920, 1080}, 2, 99999999);
    R.addFloat("World.EnvIntensityScale", {1.0}, 0.0, 100000.0);
    R.addTexture("World.Skycube"); // RVARNAME_SKYBOX: a longitude-latitude RGBA texture here
    R.addOptions("RenderPipeline", 1, {"BPT", "BPT_WITH_NEE", "BDPT", "DBG_Normals", "DBG_Tangents", "DBG_UV"});
    R.addFloat("Camera.ApertureRadius", {0.0}, 0.0, 1000.0);
    R.addFloat("Camera.FocusDistance", {10.0}, 0.001, 1000000.0);
    R.addInt("Firefly.RegularizeAfterVertices", {8}, 0, 64);
    R.addOptions("Firefly.Regularize", 1, {"OFF", "ON"});
    // tonemap stage (RendererVarsList.h:50-57) and the a-trous denoiser (RendererVarsList.h:25-32)
    R.addOptions("Tonemap.Enable", 1, {"OFF", "ON"});
    R.addFloat("Tonemap.Toe", {1.0}, 0.0, 100.0);
    R.addFloat("Tonemap.Mid", {1.0}, 0.0, 100.0);
    R.addFloat("Tonemap.Shoulder", {1.0}, 0.0, 100.0);
    R.addOptions("Tonemap.UseAutoExposure", 1, {"OFF", "ON"});
    R.addFloat("Tonemap.ExposureCompensation", {0.0}, -10000.0, 10000.0);
    R.addFloat("Tonemap.EyeAdaptationSpeed", {1.0}, 0.0, 1000.0);
    R.addFloat("Tonemap.ManualExposure", {1.0}, 0.0, 1e16);
    R.addOptions("Denoise.Mode", 0, {"OFF", "ON", "DEBUG_MAT_PARAMS", "DEBUG_VARIANCE", "DEBUG_SHOW_SAMPLE_SOURCES",
                                     "DEBUG_FEATURE_VARIANCE"});
    R.addFloat("Denoise.DepthSigmaScale", {0.02}, 0.00001, 10.0);
    R.addFloat("Denoise.NormalSigma", {0.06}, 0.00001, 1000.0);
    R.addFloat("Denoise.MaterialDifferenceSigma", {0.05}, 0.00001, 1000.0);
    R.addFloat("Denoise.ColorDifferenceSigma", {3.0}, 0.00001, 1000.0);
    R.addFloat("Denoise.FeatureVarianceScale", {1.0}, 0.0, 1000.0);
    R.addOptions("Denoise.FeaturePrefilter", 1, {"OFF", "ON"});
    R.addInt("Generic.MaxDepth", {32}, 1, 64);
    R.addInt("Generic.Seed", {0}, 0, 4294967295.0);
    R.addFloat("Generic.SpectralRange", {380.0, 700.0}, 360.0, 830.0);
    R.addInt("BDPT.LightVertices", {16}, 2, 16);
    R.addInt("BDPT.LightPaths", {0}, 0, 1 << 24);
    R.addOptions("Generic.Features", 0, {"OFF", "ON"});
}

// ------------------------------------------------------------------ scene graph
struct NodeData
{
    std::string name;
    std::shared_ptr<TransformData> transform = std::make_shared<TransformData>();
};

struct SceneObject
{
    std::shared_ptr<NodeData> node;
    std::string getName() const { return node->name; }
    Transform getTransform() const { return Transform{node->transform}; }
};

struct RenderObject : SceneObject
{
    std::shared_ptr<Mesh> mesh;
    std::vector<std::shared_ptr<Material>> materials;
    void setMesh(std::shared_ptr<Mesh> m) { mesh = std::move(m); }
    void setMaterial(std::shared_ptr<Material> m, size_t index)
    {
        if (materials.size() <= index) materials.resize(index + 1);
        materials[index] = std::move(m);
    }
    void setMaterials(std::vector<std::shared_ptr<Material>> ms) { materials = std::move(ms); }
    std::vector<std::shared_ptr<Material>> getMaterials() const { return materials; }
    std::shared_ptr<Mesh> getMesh() const { return mesh; }
};

struct Light : SceneObject
{
    LightType type = LightType::POINT;
    vec3 color{{1.f, 1.f, 1.f}};
    float intensity = 1.f;
    float inner = 0.f, outer = 0.78539816f;
    void setType(LightType t) { type = t; }
    LightType getType() const { return type; }
    void setColor(const vec3& c) { color = c; }
    vec3 getColor() const { return color; }
    void setIntensity(float i) { intensity = i; }
    float getIntensity() const { return intensity; }
    // LightProxy::setSpotConeAngles: outer clamped to [0, pi/2], inner to [0, outer]
    void setSpotConeAngles(float innerAngle, float outerAngle)
    {
        outer = std::clamp(outerAngle, 0.f, 1.57079633f);
        inner = std::clamp(innerAngle, 0.f, outer);
    }
    float getSpotInnerAngle() const { return inner; }
    float getSpotOuterAngle() const { return outer; }
};

struct CameraData
{
    float fovy = 0.94247780f; // pi * 0.3
    float aspect = 1.f, nearPlane = 0.1f, farPlane = 1000.f, orthoSize = 600.f;
    ProjectionType type = ProjectionType::PERSPECTIVE;
    std::shared_ptr<TransformData> transform = std::make_shared<TransformData>();
};

struct Camera
{
    std::shared_ptr<CameraData> d;
    void setProjectionPerspective(float fovy, float aspect, float n, float f)
    {
        d->fovy = fovy, d->aspect = aspect, d->nearPlane = n, d->farPlane = f;
        d->type = ProjectionType::PERSPECTIVE;
    }
    void setProjectionOrthographic(float size, float aspect, float n, float f)
    {
        d->orthoSize = size, d->aspect = aspect, d->nearPlane = n, d->farPlane = f;
        d->type = ProjectionType::ORTHOGRAPHIC;
    }
    void setFOVY(float v) { d->fovy = v; }
    void setAspectRatio(float v) { d->aspect = v; }
    void setNearPlane(float v) { d->nearPlane = v; }
    void setFarPlane(float v) { d->farPlane = v; }
    void setOrthographicSize(float v) { d->orthoSize = v; }
    void setProjectionType(ProjectionType t) { d->type = t; }
    float getFOVY() const { return d->fovy; }
    float getAspectRatio() const { return d->aspect; }
    float getNearPlane() const { return d->nearPlane; }
    float getFarPlane() const { return d->farPlane; }
    float getOrthographicSize() const { return d->orthoSize; }
    ProjectionType getProjectionType() const { return d->type; }
    Transform getTransform() const { return Transform{d->transform}; }

    // RaytraceConstantData matrices: view = inverse(world); glm::perspective (right handed, clip z
    // in [-1, 1]) mapped to the DX12 NDC and to texture space with v down
    // (RaytraceCommonResources.cpp:64-140, RenderAPIAbstractionUtility.h:18-58)
    yg_camera constants(float aperture, float focus) const
    {
        if (d->type != ProjectionType::PERSPECTIVE) throw YaptError("orthographic cameras are not supported");
        M4 world = d->transform->world();
        M4 view = inverse(world);
        double t = std::tan((double)d->fovy / 2.0), n = d->nearPlane, f = d->farPlane;
        M4 P{};
        P.a[0][0] = 1.0 / ((double)d->aspect * t);
        P.a[1][1] = 1.0 / t;
        P.a[2][2] = -(f + n) / (f - n);
        P.a[2][3] = -(2.0 * f * n) / (f - n);
        P.a[3][2] = -1.0;
        M4 toDx = identity();
        toDx.a[2][2] = 0.5;
        toDx.a[2][3] = 0.5;
        M4 toUv = identity();
        toUv.a[0][0] = 0.5;
        toUv.a[0][3] = 0.5;
        toUv.a[1][1] = -0.5;
        toUv.a[1][3] = 0.5;
        M4 viewToUv = mul(mul(toUv, toDx), P);
        M4 uvToView = inverse(viewToUv);
        double cz = uvToView.a[2][0] * 0.5 + uvToView.a[2][1] * 0.5 + uvToView.a[2][3];
        double cw = uvToView.a[3][0] * 0.5 + uvToView.a[3][1] * 0.5 + uvToView.a[3][3];
        yg_camera c{};
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
            {
                c.uv_to_view[4 * i + j] = (float)uvToView.a[i][j];
                c.view_to_uv[4 * i + j] = (float)viewToUv.a[i][j];
                c.world_to_view[4 * i + j] = (float)view.a[i][j];
                c.view_to_world[4 * i + j] = (float)world.a[i][j];
            }
        c.aperture_radius = std::max(0.f, aperture);
        c.focus_distance = std::max(1e-4f, focus);
        c.view_forward_z_sign = (cz / cw < 0) ? -1.f : 1.f;
        return c;
    }
};

template <typename T>
void appendBytes(std::vector<uint8_t>& out, const T& v)
{
    const uint8_t* p = reinterpret_cast<const uint8_t*>(&v);
    out.insert(out.end(), p, p + sizeof(T));
}

struct Renderer;

struct Scene
{
    std::shared_ptr<RendererState> R;
    std::vector<std::weak_ptr<RenderObject>> renderObjects;
    std::vector<std::weak_ptr<Light>> lights;
    std::vector<std::weak_ptr<SceneObject>> sceneObjects;
    std::shared_ptr<CameraData> camera = std::make_shared<CameraData>();
    double elapsed = 0;

    void init(const Renderer& r);
    void shutdown()
    {
        renderObjects.clear();
        lights.clear();
        sceneObjects.clear();
        R.reset();
    }
    void requireInit() const
    {
        if (!R || !R->ctx) throw YaptError("Scene: call init(renderer) with an initialised renderer first");
    }
    std::shared_ptr<RenderObject> createRenderObject(const std::string& name)
    {
        auto o = std::make_shared<RenderObject>();
        o->node = std::make_shared<NodeData>();
        o->node->name = name;
        renderObjects.push_back(o);
        return o;
    }
    std::shared_ptr<SceneObject> createSceneObject(const std::string& name)
    {
        auto o = std::make_shared<SceneObject>();
        o->node = std::make_shared<NodeData>();
        o->node->name = name;
        sceneObjects.push_back(o);
        return o;
    }
    std::shared_ptr<Light> createLight(const std::string& name, LightType type)
    {
        auto o = std::make_shared<Light>();
        o->node = std::make_shared<NodeData>();
        o->node->name = name;
        o->type = type;
        lights.push_back(o);
        return o;
    }
    Camera getMainCamera() const { return Camera{camera}; }

    // Commits the scene to the device when it changed; returns true when the accumulation
    // must restart.
    bool sync();
    void update(float deltaTime, uint32_t samples);
    py::dict debugRecords();
};

struct Renderer
{
    std::shared_ptr<RendererState> R;

    void init(py::object cache, uintptr_t windowHandle, bool enableGPUTrace, int device)
    {
        (void)cache;
        if (windowHandle) throw YaptError("Renderer.init: this renderer is headless (windowHandle must be 0)");
        (void)enableGPUTrace;
        shutdown();
        auto s = std::make_shared<RendererState>();
        std::string dir = packageDataDir();
        check(yg_create(dir.c_str(), device, &s->ctx), "Renderer.init");
        registerVariables(*s);
        R = s;
    }
    void shutdown() { R.reset(); }
    void requireInit() const
    {
        if (!R || !R->ctx) throw YaptError("Renderer: call init() first");
    }
    py::object getRendererVariable(const std::string& name) const
    {
        requireInit();
        for (auto& v : R->vars)
            if (v->name == name) return py::cast(RendererVariable{v, R->serial});
        return py::none();
    }
    std::vector<std::string> getAllRendererVariableNames() const
    {
        requireInit();
        std::vector<std::string> r;
        for (auto& v : R->vars) r.push_back(v->name);
        return r;
    }
    [[noreturn]] void setRenderOutputToSurface(size_t, size_t, uintptr_t)
    {
        throw YaptError("setRenderOutputToSurface: this renderer is headless; use readback()");
    }
    void resetRenderOutput() {}
    // PyRenderer::createTexture (PyRenderer.cpp:84-94): 2D, RGBA8 (UNORM / sRGB) or RGBA32 float
    Texture createTexture(const std::string& name, ResourceDimension dim, ResourceFormat fmt, uint32_t usage, uint32_t width,
                          uint32_t height, uint32_t mips, uint32_t depthOrSlices)
    {
        (void)usage;
        (void)mips;
        const bool cube = dim == ResourceDimension::TEXTURE_CUBEMAP;
        if (cube ? (depthOrSlices != 6 || width != height) : (dim != ResourceDimension::TEXTURE_2D || depthOrSlices > 1))
            throw YaptError("createTexture '" + name +
                            "': 2D textures and cube maps of six square slices are used by the GB300 integrators");
        auto t = std::make_shared<TextureData>();
        t->layers = cube ? 6 : 1;
        t->name = name;
        if (fmt == ResourceFormat::RGBA8_UNORM) t->format = YG_TEXTURE_RGBA8_UNORM;
        else if (fmt == ResourceFormat::RGBA8_SRGB) t->format = YG_TEXTURE_RGBA8_SRGB;
        else if (fmt == ResourceFormat::RGBA32_SFLOAT) t->format = YG_TEXTURE_RGBA32_FLOAT;
        else throw YaptError("createTexture '" + name + "': format must be RGBA8_UNORM, RGBA8_SRGB or RGBA32_SFLOAT");
        if (width == 0 || height == 0) throw YaptError("createTexture '" + name + "': empty texture");
        t->width = width;
        t->height = height;
        t->texels.assign((size_t)width * height * t->layers * (t->format == YG_TEXTURE_RGBA32_FLOAT ? 16 : 4), 0);
        return Texture{t};
    }
    Buffer createBuffer(const std::string& name, uint32_t usage, size_t size)
    {
        auto b = std::make_shared<BufferData>();
        b->name = name;
        b->usage = usage;
        b->bytes.assign(size, 0);
        return Buffer{b};
    }
    std::shared_ptr<Mesh> createMesh(const std::string& name, const std::vector<VertexBufferLayout>& layouts,
                                     size_t vertexCount, size_t submeshCount, bool use16)
    {
        auto d = std::make_shared<MeshData>();
        d->name = name;
        d->layouts = layouts;
        d->vertexCount = vertexCount;
        d->use16 = use16;
        d->vbuf.resize(layouts.size());
        d->vbufOffset.assign(layouts.size(), 0);
        d->submeshes.resize(submeshCount);
        return std::make_shared<Mesh>(Mesh{d});
    }
    std::shared_ptr<Material> createMaterial(const std::string& name)
    {
        auto d = std::make_shared<MaterialData>();
        d->name = name;
        setDefaults(*d);
        return std::make_shared<Material>(Material{d});
    }
    std::shared_ptr<ReadbackObject> readback(ReadbackTarget target);
    void resetAccumulation()
    {
        requireInit();
        R->frames = 0;
        R->lastParams.clear();
    }
    uint32_t getAccumulatedFrames() const { return R ? R->frames : 0; }
};

void Scene::init(const Renderer& r)
{
    r.requireInit();
    R = r.R;
}

bool Scene::sync()
{
    requireInit();
    RendererState& S = *R;
    std::vector<yg_punctual_light> punctual;
    for (auto& w : lights)
    {
        auto l = w.lock();
        if (!l) continue;
        const float k = std::max(0.f, l->intensity);
        yg_punctual_light P{};
        P.type = (uint32_t)l->type + 1u; // POINT, SPOT, DIRECTIONAL -> YG_LIGHT_*
        for (int c = 0; c < 3; ++c) P.intensity[c] = l->color.v[c] * k;
        if (P.intensity[0] == 0.f && P.intensity[1] == 0.f && P.intensity[2] == 0.f) continue;
        M4 t = l->node->transform->world();
        double d[3] = {-t.a[0][2], -t.a[1][2], -t.a[2][2]};
        double dl = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (int c = 0; c < 3; ++c)
        {
            P.position[c] = (float)t.a[c][3];
            P.direction[c] = dl > 0.0 ? (float)(d[c] / dl) : (c == 2 ? -1.f : 0.f);
        }
        P.cos_inner = std::cos(l->inner);
        P.cos_outer = std::cos(l->outer);
        punctual.push_back(P);
    }
    // gather instances in creation order (RaytraceCommonResources::sceneChanged: one instance
    // per (render object, submesh), the last material serving the submeshes beyond the list)
    std::vector<std::shared_ptr<MeshData>> meshes;
    std::vector<std::shared_ptr<MaterialData>> mats;
    std::vector<yg_instance> inst;
    auto meshIndex = [&](const std::shared_ptr<MeshData>& m) {
        for (size_t i = 0; i < meshes.size(); ++i)
            if (meshes[i] == m) return (uint32_t)i;
        meshes.push_back(m);
        return (uint32_t)meshes.size() - 1;
    };
    auto matIndex = [&](const std::shared_ptr<MaterialData>& m) {
        for (size_t i = 0; i < mats.size(); ++i)
            if (mats[i] == m) return (uint32_t)i;
        mats.push_back(m);
        return (uint32_t)mats.size() - 1;
    };
    for (auto& w : renderObjects)
    {
        auto o = w.lock();
        if (!o || !o->mesh || o->materials.empty()) continue;
        uint32_t mi = meshIndex(o->mesh->d);
        M4 o2w = o->node->transform->world();
        M4 w2o = inverse(o2w);
        for (size_t s = 0; s < o->mesh->d->submeshes.size(); ++s)
        {
            const auto& mat = s < o->materials.size() ? o->materials[s] : o->materials.back();
            if (!mat) throw YaptError("render object '" + o->node->name + "': material slot not set");
            yg_instance I{};
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 4; ++c)
                {
                    I.obj_to_world[4 * r + c] = (float)o2w.a[r][c];
                    I.world_to_obj[4 * r + c] = (float)w2o.a[r][c];
                }
            I.mesh = mi;
            I.submesh = (uint32_t)s;
            I.material = matIndex(mat->d);
            inst.push_back(I);
        }
    }
    // materials and their spectra
    std::vector<yg_material> gm;
    std::vector<float> spectra;
    auto addSpec = [&](const std::vector<float>& v) {
        if (v.empty()) return -1;
        spectra.insert(spectra.end(), v.begin(), v.end());
        return (int)(spectra.size() / kSpecPoints) - 1;
    };
    // textures in first-use order (materials, then the skybox); materials refer to id + 1
    std::vector<std::shared_ptr<TextureData>> texs;
    auto texId = [&](const std::shared_ptr<TextureData>& t) -> uint32_t {
        if (!t) return 0;
        for (size_t i = 0; i < texs.size(); ++i)
            if (texs[i] == t) return (uint32_t)i + 1;
        texs.push_back(t);
        return (uint32_t)texs.size();
    };
    for (auto& m : mats)
    {
        yg_material x = m->m;
        x.material_mask = (m->twoSided ? YG_MATERIAL_TWO_SIDED : 0u) | (m->dispersion ? YG_MATERIAL_DISPERSION : 0u) |
                          (m->alphaBlend ? YG_MATERIAL_ALPHA_BLEND : 0u);
        x.albedo_spectrum = addSpec(m->albedoSpec);
        x.specular_spectrum = addSpec(m->specularSpec);
        x.emission_spectrum = addSpec(m->emissionSpec);
        x.albedo_texture = texId(m->tex[0]);
        x.normal_texture = texId(m->tex[1]);
        x.orm_texture = texId(m->tex[2]);
        x.emissive_texture = texId(m->tex[3]);
        gm.push_back(x);
    }
    const uint32_t envTex = texId(S.var("World.Skycube")->texture);
    bool texturesChanged = false;
    std::vector<uint64_t> texSig{envTex};
    for (auto& t : texs)
    {
        texSig.push_back(reinterpret_cast<uintptr_t>(t.get()));
        texSig.push_back(t->version);
    }
    if (texSig != S.lastTextures)
    {
        check(yg_clear_textures(S.ctx), "scene update");
        for (auto& t : texs)
        {
            uint32_t id = 0;
            check(yg_upload_texture(S.ctx, t->width, t->height * t->layers, t->format, t->texels.data(), &id),
                  "scene update");
        }
        const auto& sky = S.var("World.Skycube")->texture;
        if (envTex && sky && sky->layers == 6) check(yg_set_environment_cube(S.ctx, envTex), "scene update");
        else check(yg_set_environment_texture(S.ctx, envTex), "scene update");
        S.lastTextures = texSig;
        texturesChanged = true;
    }
    std::vector<uint64_t> meshSig;
    for (auto& m : meshes)
    {
        meshSig.push_back(reinterpret_cast<uintptr_t>(m.get()));
        meshSig.push_back(m->contentVersion());
    }
    std::vector<uint8_t> sceneSig;
    for (auto& i : inst) appendBytes(sceneSig, i);
    for (auto& m : gm) appendBytes(sceneSig, m);
    for (float f : spectra) appendBytes(sceneSig, f);
    bool changed = texturesChanged;
    if (meshSig != S.lastMeshes)
    {
        check(yg_clear_meshes(S.ctx), "scene update");
        for (auto& m : meshes)
        {
            DecodedMesh dm = decodeMesh(*m);
            yg_mesh_desc d{};
            d.positions = dm.positions.data();
            d.normals = dm.normals.data();
            d.tangents = dm.hasTangents ? dm.tangents.data() : nullptr;
            d.uvs = dm.hasUvs ? dm.uvs.data() : nullptr;
            d.vertex_count = (uint32_t)m->vertexCount;
            d.indices = dm.indices.data();
            d.index_count = (uint32_t)dm.indices.size();
            d.index_bits = 32;
            d.submesh_ranges = dm.submeshes.data();
            d.submesh_count = (uint32_t)(dm.submeshes.size() / 2);
            uint32_t id = 0;
            check(yg_upload_mesh(S.ctx, &d, &id), "scene update");
        }
        S.lastMeshes = meshSig;
        S.lastScene.clear();
        changed = true;
    }
    S.instances = inst;
    S.materials = gm;
    S.spectra = spectra;
    if (sceneSig != S.lastScene || changed)
    {
        if (inst.empty()) throw YaptError("Scene.update: the scene has no render object with a mesh and a material");
        check(yg_upload_materials(S.ctx, gm.data(), (uint32_t)gm.size()), "scene update");
        check(yg_upload_spectra(S.ctx, spectra.empty() ? nullptr : spectra.data(), (uint32_t)(spectra.size() / kSpecPoints),
                                kSpecPoints, kSpecLmin, kSpecLmax),
              "scene update");
        check(yg_set_instances(S.ctx, inst.data(), (uint32_t)inst.size()), "scene update");
        check(yg_build_scene(S.ctx), "scene update");
        S.lastScene = sceneSig;
        changed = true;
    }
    std::vector<uint8_t> lightSig;
    for (auto& P : punctual) appendBytes(lightSig, P);
    if (lightSig != S.lastLights || changed)
    {
        check(yg_set_punctual_lights(S.ctx, punctual.empty() ? nullptr : punctual.data(), (uint32_t)punctual.size()),
              "scene update");
        S.lastLights = lightSig;
        changed = true;
    }
    yg_camera cam = Camera{camera}.constants((float)S.var("Camera.ApertureRadius")->val[0],
                                             (float)S.var("Camera.FocusDistance")->val[0]);
    S.camera = cam;
    std::vector<uint8_t> camSig;
    appendBytes(camSig, cam);
    if (camSig != S.lastCamera)
    {
        check(yg_set_camera(S.ctx, &cam), "scene update");
        S.lastCamera = camSig;
        changed = true;
    }
    return changed;
}

void Scene::update(float deltaTime, uint32_t samples)
{
    elapsed += deltaTime;
    bool changed = sync();
    RendererState& S = *R;
    int pipeline = S.var("RenderPipeline")->selected;
    if (pipeline > 2) throw YaptError("the debug render pipelines are not built");
    yg_render_params p{};
    p.integrator = (uint32_t)pipeline;
    p.width = (uint32_t)S.var("Generic.RenderResolution")->val[0];
    p.height = (uint32_t)S.var("Generic.RenderResolution")->val[1];
    p.max_depth = (uint32_t)S.var("Generic.MaxDepth")->val[0];
    p.regularize_after_vertices = (uint32_t)S.var("Firefly.RegularizeAfterVertices")->val[0];
    p.regularize_enable = (uint32_t)S.var("Firefly.Regularize")->selected;
    p.env_intensity_scale = (float)S.var("World.EnvIntensityScale")->val[0];
    p.seed = (uint32_t)S.var("Generic.Seed")->val[0];
    p.lambda_min = (float)S.var("Generic.SpectralRange")->val[0];
    p.lambda_max = (float)S.var("Generic.SpectralRange")->val[1];
    p.bdpt_light_vertices = (uint32_t)S.var("BDPT.LightVertices")->val[0];
    p.bdpt_light_paths = (uint32_t)S.var("BDPT.LightPaths")->val[0];
    bool feats = S.var("Generic.Features")->selected == 1;
    const int denoise = S.var("Denoise.Mode")->selected;
    if (denoise > 1) throw YaptError("Denoise.Mode: only OFF and ON are built (the debug views are not)");
    p.flags = (feats ? YG_FLAG_FEATURES : 0u) | (denoise == 1 ? YG_FLAG_ATROUS_FEATURES : 0u);
    S.lastDeltaTime = deltaTime;
    std::vector<uint8_t> sig;
    appendBytes(sig, p);
    if (changed || sig != S.lastParams || p.width != S.filmW || p.height != S.filmH)
    {
        check(yg_film_clear(S.ctx, p.width, p.height), "Scene.update");
        S.frames = 0;
        S.filmW = p.width;
        S.filmH = p.height;
        S.lastParams = sig;
    }
    S.featuresOn = feats;
    if (samples == 0) return;
    p.spp_start = S.frames;
    p.spp_count = samples;
    check(yg_render(S.ctx, &p, nullptr), "Scene.update");
    S.frames += samples;
}

py::dict Scene::debugRecords()
{
    requireInit();
    sync();
    auto bytesOf = [](const void* p, size_t n) { return py::bytes(reinterpret_cast<const char*>(p), n); };
    py::dict d;
    d["camera"] = bytesOf(&R->camera, sizeof(yg_camera));
    d["instances"] = bytesOf(R->instances.data(), R->instances.size() * sizeof(yg_instance));
    d["materials"] = bytesOf(R->materials.data(), R->materials.size() * sizeof(yg_material));
    d["spectra"] = bytesOf(R->spectra.data(), R->spectra.size() * sizeof(float));
    return d;
}

std::shared_ptr<ReadbackObject> Renderer::readback(ReadbackTarget target)
{
    requireInit();
    RendererState& S = *R;
    auto ro = std::make_shared<ReadbackObject>();
    if (S.filmW == 0)
    {
        ro->state = ReadbackState::Failed;
        return ro;
    }
    const size_t n = (size_t)S.filmW * S.filmH;
    auto data = std::make_shared<ReadbackData>();
    data->width = S.filmW;
    data->height = S.filmH;
    std::vector<float> xyz(n * 3), cnt(n);
    if (target == ReadbackTarget::Features)
    {
        if (!S.featuresOn)
        {
            ro->state = ReadbackState::Failed;
            return ro;
        }
        std::vector<float> alb(n * 3), nrm(n * 3), dep(n);
        check(yg_features_read(S.ctx, alb.data(), nrm.data(), dep.data()), "readback");
        data->format = ResourceFormat::RGBA32_SFLOAT;
        data->slices = 2;
        data->bytes.resize(n * 32);
        float* o = reinterpret_cast<float*>(data->bytes.data());
        for (size_t i = 0; i < n; ++i)
        {
            o[4 * i] = alb[3 * i], o[4 * i + 1] = alb[3 * i + 1], o[4 * i + 2] = alb[3 * i + 2], o[4 * i + 3] = dep[i];
            float* q = o + 4 * n + 4 * i;
            q[0] = nrm[3 * i], q[1] = nrm[3 * i + 1], q[2] = nrm[3 * i + 2], q[3] = 0.f;
        }
        ro->data = data;
        ro->state = ReadbackState::Ready;
        return ro;
    }
    check(yg_film_read(S.ctx, xyz.data(), cnt.data()), "readback");
    // c_srgbXYZToRGB (colorSpaces.hlsl:18-23)
    const float M[3][3] = {{3.2406f, -1.5372f, -0.4986f}, {-0.9689f, 1.8758f, 0.0415f}, {0.0557f, -0.2040f, 1.0570f}};
    auto rgbOf = [&](size_t i, float out[3]) {
        for (int r = 0; r < 3; ++r)
            out[r] = M[r][0] * xyz[3 * i] + M[r][1] * xyz[3 * i + 1] + M[r][2] * xyz[3 * i + 2];
    };
    if (target == ReadbackTarget::FinalColor)
    {
        // the combine stage's a-trous denoiser when Denoise.Mode is ON, then the tonemap stage
        data->format = ResourceFormat::RGBA8_UNORM;
        data->bytes.resize(n * 4);
        const bool denoise = S.var("Denoise.Mode")->selected == 1;
        if (denoise)
        {
            yg_atrous_params a;
            yg_atrous_default_params(&a);
            a.depth_sigma_scale = (float)S.var("Denoise.DepthSigmaScale")->val[0];
            a.normal_sigma = (float)S.var("Denoise.NormalSigma")->val[0];
            a.material_sigma = (float)S.var("Denoise.MaterialDifferenceSigma")->val[0];
            a.color_sigma = (float)S.var("Denoise.ColorDifferenceSigma")->val[0];
            a.feature_variance_scale = (float)S.var("Denoise.FeatureVarianceScale")->val[0];
            a.prefilter = (uint32_t)S.var("Denoise.FeaturePrefilter")->selected;
            check(yg_atrous_denoise(S.ctx, &a, nullptr, nullptr), "readback");
        }
        yg_tonemap_params t;
        yg_tonemap_default_params(&t);
        t.enable = (uint32_t)S.var("Tonemap.Enable")->selected;
        t.auto_exposure = (uint32_t)S.var("Tonemap.UseAutoExposure")->selected;
        t.manual_exposure = (float)S.var("Tonemap.ManualExposure")->val[0];
        t.exposure_compensation = (float)S.var("Tonemap.ExposureCompensation")->val[0];
        t.eye_adaptation_speed = (float)S.var("Tonemap.EyeAdaptationSpeed")->val[0];
        t.delta_time = S.lastDeltaTime;
        t.reset = S.tonemapStarted ? 0u : 1u;
        t.source = denoise ? 1u : 0u;
        check(yg_tonemap(S.ctx, &t, data->bytes.data(), nullptr), "readback");
        S.tonemapStarted = true;
    }
    else
    {
        data->format = ResourceFormat::RGBA32_SFLOAT;
        data->bytes.resize(n * 16);
        float* o = reinterpret_cast<float*>(data->bytes.data());
        for (size_t i = 0; i < n; ++i)
        {
            if (target == ReadbackTarget::FilmXYZ)
            {
                o[4 * i] = xyz[3 * i], o[4 * i + 1] = xyz[3 * i + 1], o[4 * i + 2] = xyz[3 * i + 2];
            }
            else
            {
                rgbOf(i, o + 4 * i);
            }
            o[4 * i + 3] = cnt[i];
        }
    }
    ro->data = data;
    ro->state = ReadbackState::Ready;
    return ro;
}

} // namespace pyyapt

PYBIND11_MODULE(py_yapt, m)
{
    using namespace pyyapt;
    m.doc() = "YAPT's Python module surface over the GB300 integrators (headless)";
    py::register_exception<YaptError>(m, "YaptError", PyExc_RuntimeError);

    bindVec<float, 2>(m, "vec2");
    bindVec<float, 3>(m, "vec3");
    bindVec<float, 4>(m, "vec4");
    bindVec<int32_t, 2>(m, "ivec2");
    bindVec<int32_t, 3>(m, "ivec3");
    bindVec<int32_t, 4>(m, "ivec4");

    py::enum_<AttributeSemanticName>(m, "AttributeSemanticName")
        .value("UNKNOWN", AttributeSemanticName::UNKNOWN)
        .value("POSITION", AttributeSemanticName::POSITION)
        .value("TEXCOORD", AttributeSemanticName::TEXCOORD)
        .value("NORMAL", AttributeSemanticName::NORMAL)
        .value("TANGENT", AttributeSemanticName::TANGENT)
        .value("COLOR", AttributeSemanticName::COLOR);
    py::enum_<ResourceDimension>(m, "ResourceDimension")
        .value("BUFFER", ResourceDimension::BUFFER)
        .value("TEXTURE_1D", ResourceDimension::TEXTURE_1D)
        .value("TEXTURE_1D_ARRAY", ResourceDimension::TEXTURE_1D_ARRAY)
        .value("TEXTURE_2D", ResourceDimension::TEXTURE_2D)
        .value("TEXTURE_2D_ARRAY", ResourceDimension::TEXTURE_2D_ARRAY)
        .value("TEXTURE_3D", ResourceDimension::TEXTURE_3D)
        .value("TEXTURE_CUBEMAP", ResourceDimension::TEXTURE_CUBEMAP)
        .value("TEXTURE_CUBEMAP_ARRAY", ResourceDimension::TEXTURE_CUBEMAP_ARRAY)
        .value("UNDEFINED", ResourceDimension::UNDEFINED);
    {
        py::enum_<ResourceFormat> e(m, "ResourceFormat");
#define YG_VALUE(n, s) e.value(#n, ResourceFormat::n);
        YG_FORMATS(YG_VALUE)
#undef YG_VALUE
    }
    py::enum_<ResourceUsageBits>(m, "ResourceUsageBits", py::arithmetic())
        .value("UNKNOWN", RESOURCE_USAGE_UNKNOWN)
        .value("COPY_DESTINATION", RESOURCE_USAGE_COPY_DESTINATION)
        .value("COPY_SOURCE", RESOURCE_USAGE_COPY_SOURCE)
        .value("UNIFORM_BUFFER", RESOURCE_USAGE_UNIFORM_BUFFER)
        .value("STORAGE_BUFFER", RESOURCE_USAGE_STORAGE_BUFFER)
        .value("VERTEX_BUFFER", RESOURCE_USAGE_VERTEX_BUFFER)
        .value("INDEX_BUFFER", RESOURCE_USAGE_INDEX_BUFFER)
        .value("ACCELERATION_STRUCTURE_BUILD_INPUT", RESOURCE_USAGE_ACCELERATION_STRUCTURE_BUILD_INPUT)
        .value("SAMPLED_TEXTURE", RESOURCE_USAGE_SAMPLED_TEXTURE)
        .value("STORAGE_TEXTURE", RESOURCE_USAGE_STORAGE_TEXTURE)
        .export_values();

    py::class_<RendererCacheTag>(m, "RendererCache")
        .def_static("getDefaultRendererCache", []() { return RendererCacheTag{}; });

    py::class_<Transform>(m, "Transform")
        .def("setTranslation", &Transform::setTranslation)
        .def("addTranslation", &Transform::addTranslation)
        .def("getTranslation", &Transform::getTranslation)
        .def("setScale", &Transform::setScale)
        .def("addScale", &Transform::addScale)
        .def("getScale", &Transform::getScale)
        .def("setOrientation", &Transform::setOrientation)
        .def("addOrientation", &Transform::addOrientation)
        .def("getOrientation", &Transform::getOrientation)
        .def("lookAt", &Transform::lookAt)
        .def("right", [](const Transform& t) { return t.axis(1, 0, 0); })
        .def("up", [](const Transform& t) { return t.axis(0, 1, 0); })
        .def("forward", [](const Transform& t) { return t.axis(0, 0, -1); })
        .def("setParent", &Transform::setParent)
        .def("getId", &Transform::getId)
        .def("getParentId", &Transform::getParentId)
        .def("getMatrixWS", &Transform::getMatrixWS);

    py::class_<Buffer>(m, "Buffer").def("upload", &Buffer::upload).def("getName", &Buffer::getName);

    py::class_<MeshAttribute>(m, "MeshAttribute")
        .def(py::init<>())
        .def(py::init([](ResourceFormat f, AttributeSemanticName s, uint32_t i) { return MeshAttribute{f, s, i, 0xFFFFFFFFu}; }))
        .def(py::init([](ResourceFormat f, AttributeSemanticName s, uint32_t i, uint32_t o) { return MeshAttribute{f, s, i, o}; }))
        .def_readwrite("format", &MeshAttribute::format)
        .def_readwrite("semanticName", &MeshAttribute::semanticName)
        .def_readwrite("semanticIndex", &MeshAttribute::semanticIndex)
        .def_readwrite("offset", &MeshAttribute::offset);
    py::class_<VertexBufferLayout>(m, "VertexBufferLayout")
        .def(py::init<>())
        .def(py::init([](std::vector<MeshAttribute> a, uint32_t stride) { return VertexBufferLayout{std::move(a), stride}; }))
        .def_readwrite("attributes", &VertexBufferLayout::attributes)
        .def_readwrite("vertexStrideInBytes", &VertexBufferLayout::vertexStrideInBytes)
        .def_readonly_static("STRIDE_TIGHTLY_PACKED", &VertexBufferLayout::STRIDE_TIGHTLY_PACKED);
    py::class_<Mesh, std::shared_ptr<Mesh>>(m, "Mesh")
        .def("getName", &Mesh::getName)
        .def("setVertexBuffer", &Mesh::setVertexBuffer)
        .def("setIndexBuffer", &Mesh::setIndexBuffer)
        .def("setSubmesh", &Mesh::setSubmesh)
        .def("getSubmeshCount", &Mesh::getSubmeshCount)
        .def("_decoded", &Mesh::decoded)
        .def_static("calculateBoundsFromVertexBuffer", &calculateBounds);

    auto mat = py::class_<Material, std::shared_ptr<Material>>(m, "Material");
    mat.def("setFromMaterialPreset", &Material::setFromMaterialPreset)
        .def("getName", &Material::getName)
#define YG_PROP(N) .def("set" #N, &Material::set##N).def("get" #N, &Material::get##N)
        YG_PROP(Transparency) YG_PROP(Metalness) YG_PROP(Albedo) YG_PROP(SpecularTint) YG_PROP(Absorption)
        YG_PROP(Emission) YG_PROP(EmissionFocus) YG_PROP(DielectricIOR) YG_PROP(Roughness) YG_PROP(Anisotropy)
        YG_PROP(AnisotropyRotation) YG_PROP(TwoSided) YG_PROP(SpecularAmount) YG_PROP(ClearCoatAmount)
        YG_PROP(ClearCoatRoughness) YG_PROP(ClearCoatIOR) YG_PROP(SheenRoughness) YG_PROP(SheenTint)
        YG_PROP(SheenAmount) YG_PROP(AlphaCutoff) YG_PROP(AlphaBlend) YG_PROP(ThinFilmThicknessNM)
        YG_PROP(CauchysCoefficients) YG_PROP(EnableDispersion) YG_PROP(SubsurfaceAmount) YG_PROP(SubsurfaceRadius)
        YG_PROP(SubsurfaceRadiusScale)
#undef YG_PROP
        .def("setAlbedoTexture", [](Material& m, const Texture& t, const vec2& s) { m.setSlot(0, t.d, s); }, py::arg("texture"),
             py::arg("scale") = vec2{{1.f, 1.f}})
        .def("setNormalTexture", [](Material& m, const Texture& t, const vec2& s) { m.setSlot(1, t.d, s); }, py::arg("texture"),
             py::arg("scale") = vec2{{1.f, 1.f}})
        .def("setORMTexture", [](Material& m, const Texture& t, const vec2& s) { m.setSlot(2, t.d, s); }, py::arg("texture"),
             py::arg("scale") = vec2{{1.f, 1.f}})
        .def("setEmissiveTexture", [](Material& m, const Texture& t, const vec2& s) { m.setSlot(3, t.d, s); },
             py::arg("texture"), py::arg("scale") = vec2{{1.f, 1.f}})
        .def("setAlbedoSpectrum", &Material::setAlbedoSpectrum)
        .def("setSpecularSpectrum", &Material::setSpecularSpectrum)
        .def("setEmissionSpectrum", &Material::setEmissionSpectrum)
        .def("setEmissionBlackbody", &Material::setEmissionBlackbody)
        .def("getAlbedoSpectrum", &Material::getAlbedoSpectrum)
        .def("getEmissionSpectrum", &Material::getEmissionSpectrum);
    py::enum_<MaterialPreset>(mat, "MaterialPreset")
        .value("BLANK", MaterialPreset::BLANK)
        .value("METAL_GOLD", MaterialPreset::METAL_GOLD)
        .value("METAL_SILVER", MaterialPreset::METAL_SILVER)
        .value("METAL_COPPER", MaterialPreset::METAL_COPPER)
        .value("METAL_BRASS", MaterialPreset::METAL_BRASS)
        .value("METAL_ALUMINIUM", MaterialPreset::METAL_ALUMINIUM)
        .value("GLASS", MaterialPreset::GLASS)
        .value("PLASTIC", MaterialPreset::PLASTIC)
        .export_values();

    py::class_<SceneObject, std::shared_ptr<SceneObject>>(m, "SceneObject")
        .def("getName", &SceneObject::getName)
        .def("getTransform", &SceneObject::getTransform);
    py::class_<RenderObject, SceneObject, std::shared_ptr<RenderObject>>(m, "RenderObject")
        .def("setMesh", &RenderObject::setMesh)
        .def("setMaterial", &RenderObject::setMaterial)
        .def("setMaterials", &RenderObject::setMaterials)
        .def("getMaterials", &RenderObject::getMaterials)
        .def("getMesh", &RenderObject::getMesh);
    auto light = py::class_<Light, SceneObject, std::shared_ptr<Light>>(m, "Light");
    light.def("setType", &Light::setType)
        .def("getType", &Light::getType)
        .def("setColor", &Light::setColor)
        .def("getColor", &Light::getColor)
        .def("setIntensity", &Light::setIntensity)
        .def("getIntensity", &Light::getIntensity)
        .def("setSpotConeAngles", &Light::setSpotConeAngles)
        .def("getSpotInnerAngle", &Light::getSpotInnerAngle)
        .def("getSpotOuterAngle", &Light::getSpotOuterAngle);
    py::enum_<LightType>(light, "LightType")
        .value("POINT", LightType::POINT)
        .value("SPOT", LightType::SPOT)
        .value("DIRECTIONAL", LightType::DIRECTIONAL)
        .export_values();

    auto cam = py::class_<Camera>(m, "Camera");
    cam.def("setProjectionPerspective", &Camera::setProjectionPerspective)
        .def("setProjectionOrthographic", &Camera::setProjectionOrthographic)
        .def("setFOVY", &Camera::setFOVY)
        .def("setAspectRatio", &Camera::setAspectRatio)
        .def("setNearPlane", &Camera::setNearPlane)
        .def("setFarPlane", &Camera::setFarPlane)
        .def("setOrthographicSize", &Camera::setOrthographicSize)
        .def("setProjectionType", &Camera::setProjectionType)
        .def("getFOVY", &Camera::getFOVY)
        .def("getAspectRatio", &Camera::getAspectRatio)
        .def("getNearPlane", &Camera::getNearPlane)
        .def("getFarPlance", &Camera::getFarPlane) // the reference's spelling
        .def("getFarPlane", &Camera::getFarPlane)
        .def("getOrthographicSize", &Camera::getOrthographicSize)
        .def("getProjectionType", &Camera::getProjectionType)
        .def("getTransform", &Camera::getTransform)
        .def("_constants", [](const Camera& c, float aperture, float focus) {
            yg_camera k = c.constants(aperture, focus);
            py::dict r;
            r["uv_to_view"] = std::vector<float>(k.uv_to_view, k.uv_to_view + 16);
            r["view_to_uv"] = std::vector<float>(k.view_to_uv, k.view_to_uv + 16);
            r["world_to_view"] = std::vector<float>(k.world_to_view, k.world_to_view + 16);
            r["view_to_world"] = std::vector<float>(k.view_to_world, k.view_to_world + 16);
            r["z_sign"] = k.view_forward_z_sign;
            return r;
        });
    py::enum_<ProjectionType>(cam, "ProjectionType")
        .value("PERSPECTIVE", ProjectionType::PERSPECTIVE)
        .value("ORTHOGRAPHIC", ProjectionType::ORTHOGRAPHIC)
        .export_values();

    py::enum_<RendererVariableType>(m, "RendererVariableType")
        .value("FLOAT", RendererVariableType::FLOAT)
        .value("INT", RendererVariableType::INT)
        .value("TEXTURE", RendererVariableType::TEXTURE)
        .value("BUFFER", RendererVariableType::BUFFER)
        .value("OPTIONS", RendererVariableType::OPTIONS);
    py::class_<RendererVariable>(m, "RendererVariable")
        .def("setFromFloatArray", &RendererVariable::setFromFloatArray)
        .def("setFromIntArray", &RendererVariable::setFromIntArray)
        .def("getAsFloatArray", &RendererVariable::getAsFloatArray)
        .def("getAsIntArray", &RendererVariable::getAsIntArray)
        .def("getLimitsFloat", &RendererVariable::getLimitsFloat)
        .def("getLimitsInt", &RendererVariable::getLimitsInt)
        .def("getComponentCount", &RendererVariable::getComponentCount)
        .def("getOptions", &RendererVariable::getOptions)
        .def("getSelectedOption", &RendererVariable::getSelectedOption)
        .def("setSelectedOption", &RendererVariable::setSelectedOption)
        .def("getType", &RendererVariable::getType)
        .def("setTexture", &RendererVariable::setTexture)
        .def("getTexture", &RendererVariable::getTexture);
    py::class_<Texture>(m, "Texture").def("upload", &Texture::upload).def("getName", &Texture::getName);

    py::enum_<ReadbackTarget>(m, "ReadbackTarget")
        .value("FinalColor", ReadbackTarget::FinalColor)
        .value("FilmXYZ", ReadbackTarget::FilmXYZ)
        .value("FilmRGB", ReadbackTarget::FilmRGB)
        .value("Features", ReadbackTarget::Features);
    py::enum_<ReadbackState>(m, "ReadbackState")
        .value("Created", ReadbackState::Created)
        .value("Pending", ReadbackState::Pending)
        .value("Ready", ReadbackState::Ready)
        .value("Failed", ReadbackState::Failed)
        .value("Freed", ReadbackState::Freed);
    py::class_<ReadbackData, std::shared_ptr<ReadbackData>>(m, "ReadbackData")
        .def("getWidth", [](const ReadbackData& d) { return d.width; })
        .def("getHeight", [](const ReadbackData& d) { return d.height; })
        .def("getDepthOrSlices", [](const ReadbackData& d) { return d.slices; })
        .def("getTexelSizeInBytes", [](const ReadbackData& d) { return d.texel(); })
        .def("getRowPitchInBytes", [](const ReadbackData& d) { return d.width * d.texel(); })
        .def("getSizeInBytes", [](const ReadbackData& d) { return d.bytes.size(); })
        .def("getFormat", [](const ReadbackData& d) { return d.format; })
        .def("getDimensions", [](const ReadbackData&) { return ResourceDimension::TEXTURE_2D; })
        .def("getBytes", [](const ReadbackData& d) {
            return py::bytes(reinterpret_cast<const char*>(d.bytes.data()), d.bytes.size());
        });
    py::class_<ReadbackObject, std::shared_ptr<ReadbackObject>>(m, "ReadbackObject")
        .def("getState", &ReadbackObject::getState)
        .def("isReady", &ReadbackObject::isReady)
        .def("release", &ReadbackObject::release)
        .def("getData", &ReadbackObject::getData);

    py::class_<Renderer>(m, "Renderer")
        .def(py::init<>())
        .def("init", &Renderer::init, py::arg("cache") = py::none(), py::arg("windowHandle") = 0,
             py::arg("enableGPUTrace") = false, py::arg("device") = 0)
        .def("shutdown", &Renderer::shutdown)
        .def("getRendererVariable", &Renderer::getRendererVariable)
        .def("getAllRendererVariableNames", &Renderer::getAllRendererVariableNames)
        .def("setRenderOutputToSurface", &Renderer::setRenderOutputToSurface)
        .def("resetRenderOutput", &Renderer::resetRenderOutput)
        .def("createTexture", &Renderer::createTexture)
        .def("createBuffer", &Renderer::createBuffer)
        .def("createMesh", &Renderer::createMesh)
        .def("createMaterial", &Renderer::createMaterial)
        .def("readback", &Renderer::readback)
        .def("resetAccumulation", &Renderer::resetAccumulation)
        .def("getAccumulatedFrames", &Renderer::getAccumulatedFrames);

    py::class_<Scene>(m, "Scene")
        .def(py::init<>())
        .def("init", &Scene::init)
        .def("shutdown", &Scene::shutdown)
        .def("update", &Scene::update, py::arg("deltaTime") = 0.f, py::arg("samples") = 1u)
        .def("createRenderObject", &Scene::createRenderObject)
        .def("createSceneObject", &Scene::createSceneObject)
        .def("createLight", &Scene::createLight)
        .def("getMainCamera", &Scene::getMainCamera)
        .def("_debugRecords", &Scene::debugRecords);
}
