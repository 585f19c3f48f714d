// Stand-in for the subset of the Embree 4 API that the antipodal reference uses, so that its Embree-gated
// code (RobustMeshGwn in src/antipodal/gwn_mesh_robust.hh, EmbreeIntersector in
// src/antipodal/intersector/intersector_embree.hh) compiles in a container without Embree.
//
// TEST INFRASTRUCTURE ONLY: it is used to build oracle/_ref, the reference compiled from its own sources,
// which pins the CPU restatement in oracle/gwn_oracle.cc.  It is a project-written linear scan, not Embree:
//  - user geometry: rtcOccluded1 calls the occluded callback once for every primitive.  The reference's
//    callback decides each crossing with its own exact predicate; Embree's boxes only cull candidates,
//    conservatively (gwn_mesh_robust.hh:82-90), so visiting every primitive yields the same count.
//  - triangle geometry: each triangle is tested with a float Moller-Trumbore and every hit is handed to the
//    argument filter with its geometric normal, in primitive order.  This makes EmbreeIntersector compile
//    and run; its counts are a plain float crossing count, not a bit-for-bit copy of Embree's.
// Only the names and the calling convention follow Embree's public API; the bodies are our own.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <vector>

struct RTCDeviceTy;
struct RTCSceneTy;
struct RTCGeometryTy;

enum RTCGeometryType
{
    RTC_GEOMETRY_TYPE_TRIANGLE = 0,
    RTC_GEOMETRY_TYPE_USER = 120
};
enum RTCBufferType
{
    RTC_BUFFER_TYPE_INDEX = 0,
    RTC_BUFFER_TYPE_VERTEX = 1
};
enum RTCFormat
{
    RTC_FORMAT_UINT3 = 0x5003,
    RTC_FORMAT_FLOAT3 = 0x9003
};
enum RTCBuildQuality
{
    RTC_BUILD_QUALITY_LOW = 0,
    RTC_BUILD_QUALITY_MEDIUM = 1,
    RTC_BUILD_QUALITY_HIGH = 2
};
enum RTCSceneFlags
{
    RTC_SCENE_FLAG_NONE = 0,
    RTC_SCENE_FLAG_ROBUST = 1 << 2
};
enum RTCRayQueryFlags
{
    RTC_RAY_QUERY_FLAG_NONE = 0,
    RTC_RAY_QUERY_FLAG_INVOKE_ARGUMENT_FILTER = 1 << 1,
    RTC_RAY_QUERY_FLAG_COHERENT = 1 << 0
};
enum RTCFeatureFlags : unsigned
{
    RTC_FEATURE_FLAG_NONE = 0,
    RTC_FEATURE_FLAG_ALL = 0xffffffffu
};

struct RTCRayQueryContext
{
    unsigned instID[1];
};

struct RTCRay
{
    float org_x, org_y, org_z, tnear;
    float dir_x, dir_y, dir_z, time;
    float tfar;
    unsigned mask, id, flags;
};

struct RTCHit
{
    float Ng_x, Ng_y, Ng_z;
    float u, v;
    unsigned primID, geomID;
    unsigned instID[1];
};

struct RTCRayN;
struct RTCHitN;

struct RTCBounds
{
    float lower_x, lower_y, lower_z, align0;
    float upper_x, upper_y, upper_z, align1;
};

struct RTCBoundsFunctionArguments
{
    void* geometryUserPtr;
    unsigned primID;
    unsigned timeStep;
    RTCBounds* bounds_o;
};
typedef void (*RTCBoundsFunction)(RTCBoundsFunctionArguments const* args);

struct RTCOccludedFunctionNArguments
{
    int* valid;
    void* geometryUserPtr;
    unsigned primID;
    RTCRayQueryContext* context;
    RTCRayN* ray;
    unsigned N;
    unsigned geomID;
};
typedef void (*RTCOccludedFunctionN)(RTCOccludedFunctionNArguments const* args);

struct RTCFilterFunctionNArguments
{
    int* valid;
    void* geometryUserPtr;
    RTCRayQueryContext* context;
    RTCRayN* ray;
    RTCHitN* hit;
    unsigned N;
};
typedef void (*RTCFilterFunctionN)(RTCFilterFunctionNArguments const* args);

struct RTCOccludedArguments
{
    RTCRayQueryFlags flags;
    RTCFeatureFlags feature_mask;
    RTCRayQueryContext* context;
    RTCFilterFunctionN filter;
    RTCOccludedFunctionN occluded;
};

struct RTCGeometryTy
{
    RTCGeometryType type;
    int refs = 1;
    // triangle geometry
    float const* vertex = nullptr;
    std::size_t vertex_stride = 0;
    unsigned const* index = nullptr;
    std::size_t index_stride = 0;
    std::size_t tri_count = 0;
    // user geometry
    unsigned prim_count = 0;
    void* user = nullptr;
    RTCBoundsFunction bounds = nullptr;
    RTCOccludedFunctionN occluded = nullptr;
};

struct RTCSceneTy
{
    std::vector<RTCGeometryTy*> geoms;
};

struct RTCDeviceTy
{
    int unused = 0;
};

typedef RTCDeviceTy* RTCDevice;
typedef RTCSceneTy* RTCScene;
typedef RTCGeometryTy* RTCGeometry;

inline RTCDevice rtcNewDevice(char const*)
{
    return new RTCDeviceTy{};
}
inline void rtcReleaseDevice(RTCDevice d)
{
    delete d;
}
inline RTCScene rtcNewScene(RTCDevice)
{
    return new RTCSceneTy{};
}
inline void rtcReleaseGeometry(RTCGeometry g)
{
    if (g && --g->refs == 0)
        delete g;
}
inline void rtcReleaseScene(RTCScene s)
{
    if (!s)
        return;
    for (auto* g : s->geoms)
        rtcReleaseGeometry(g);
    delete s;
}
inline void rtcSetSceneBuildQuality(RTCScene, RTCBuildQuality) {}
inline void rtcSetSceneFlags(RTCScene, RTCSceneFlags) {}
inline void rtcCommitScene(RTCScene) {}
inline RTCGeometry rtcNewGeometry(RTCDevice, RTCGeometryType type)
{
    auto* g = new RTCGeometryTy{};
    g->type = type;
    return g;
}
inline void rtcSetSharedGeometryBuffer(RTCGeometry g, RTCBufferType type, unsigned, RTCFormat, void const* ptr,
                                       std::size_t byte_offset, std::size_t byte_stride, std::size_t count)
{
    auto const* base = static_cast<unsigned char const*>(ptr) + byte_offset;
    if (type == RTC_BUFFER_TYPE_VERTEX)
    {
        g->vertex = reinterpret_cast<float const*>(base);
        g->vertex_stride = byte_stride;
    }
    else
    {
        g->index = reinterpret_cast<unsigned const*>(base);
        g->index_stride = byte_stride;
        g->tri_count = count;
    }
}
inline void rtcSetGeometryUserPrimitiveCount(RTCGeometry g, unsigned n)
{
    g->prim_count = n;
}
inline void rtcSetGeometryUserData(RTCGeometry g, void* p)
{
    g->user = p;
}
inline void rtcSetGeometryBoundsFunction(RTCGeometry g, RTCBoundsFunction f, void*)
{
    g->bounds = f;
}
inline void rtcSetGeometryOccludedFunction(RTCGeometry g, RTCOccludedFunctionN f)
{
    g->occluded = f;
}
inline void rtcCommitGeometry(RTCGeometry) {}
inline unsigned rtcAttachGeometry(RTCScene s, RTCGeometry g)
{
    ++g->refs;
    s->geoms.push_back(g);
    return unsigned(s->geoms.size() - 1);
}
inline void rtcInitRayQueryContext(RTCRayQueryContext* c)
{
    c->instID[0] = ~0u;
}
inline void rtcInitOccludedArguments(RTCOccludedArguments* a)
{
    a->flags = RTC_RAY_QUERY_FLAG_NONE;
    a->feature_mask = RTC_FEATURE_FLAG_ALL;
    a->context = nullptr;
    a->filter = nullptr;
    a->occluded = nullptr;
}

namespace fake_embree_detail
{
inline void vtx(RTCGeometryTy const* g, unsigned i, float out[3])
{
    auto const* p = reinterpret_cast<float const*>(reinterpret_cast<unsigned char const*>(g->vertex)
                                                   + std::size_t(i) * g->vertex_stride);
    out[0] = p[0];
    out[1] = p[1];
    out[2] = p[2];
}
} // namespace fake_embree_detail

inline void rtcOccluded1(RTCScene s, RTCRay* ray, RTCOccludedArguments* args)
{
    namespace fd = fake_embree_detail;
    for (unsigned gid = 0; gid < s->geoms.size(); ++gid)
    {
        RTCGeometryTy const* g = s->geoms[gid];
        if (g->type == RTC_GEOMETRY_TYPE_USER)
        {
            for (unsigned prim = 0; prim < g->prim_count; ++prim)
            {
                int valid = -1;
                RTCOccludedFunctionNArguments oa{&valid, g->user, prim, args->context,
                                                 reinterpret_cast<RTCRayN*>(ray), 1, gid};
                g->occluded(&oa);
            }
        }
        else
        {
            float const d[3] = {ray->dir_x, ray->dir_y, ray->dir_z};
            float const o[3] = {ray->org_x, ray->org_y, ray->org_z};
            for (std::size_t t = 0; t < g->tri_count; ++t)
            {
                auto const* ix = reinterpret_cast<unsigned const*>(reinterpret_cast<unsigned char const*>(g->index)
                                                                   + t * g->index_stride);
                float a[3], b[3], c[3];
                fd::vtx(g, ix[0], a);
                fd::vtx(g, ix[1], b);
                fd::vtx(g, ix[2], c);
                float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
                float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
                float h[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
                float const det = e1[0] * h[0] + e1[1] * h[1] + e1[2] * h[2];
                if (det == 0.0f)
                    continue;
                float const inv = 1.0f / det;
                float sv[3] = {o[0] - a[0], o[1] - a[1], o[2] - a[2]};
                float const u = inv * (sv[0] * h[0] + sv[1] * h[1] + sv[2] * h[2]);
                if (u < 0.0f || u > 1.0f)
                    continue;
                float q[3] = {sv[1] * e1[2] - sv[2] * e1[1], sv[2] * e1[0] - sv[0] * e1[2],
                              sv[0] * e1[1] - sv[1] * e1[0]};
                float const v = inv * (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]);
                if (v < 0.0f || u + v > 1.0f)
                    continue;
                float const th = inv * (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]);
                if (th < ray->tnear || th > ray->tfar)
                    continue;
                RTCHit hit{};
                hit.Ng_x = e1[1] * e2[2] - e1[2] * e2[1];
                hit.Ng_y = e1[2] * e2[0] - e1[0] * e2[2];
                hit.Ng_z = e1[0] * e2[1] - e1[1] * e2[0];
                hit.u = u;
                hit.v = v;
                hit.primID = unsigned(t);
                hit.geomID = gid;
                int valid = -1;
                if (args->filter)
                {
                    RTCFilterFunctionNArguments fa{&valid, nullptr, args->context, reinterpret_cast<RTCRayN*>(ray),
                                                   reinterpret_cast<RTCHitN*>(&hit), 1};
                    args->filter(&fa);
                }
                if (valid != 0)
                {
                    ray->tfar = -std::numeric_limits<float>::infinity();
                    return;
                }
            }
        }
    }
}
