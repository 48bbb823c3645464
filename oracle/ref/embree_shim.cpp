// Brute-force stand-in for the 13 Embree 2.17 entry points the reference calls
// (src/scene.cpp:42-111, src/trianglemesh.cpp:107-141). Embree's own sources need
// Embree's cmake build, so the oracle build of the reference links this instead:
// closest hit = exact double-precision Moller-Trumbore over every triangle of
// every mesh, any-hit for occlusion. Test infrastructure, never shipped.
#include <embree2/rtcore.h>
#include <embree2/rtcore_ray.h>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {
struct ShimMesh {
    std::vector<float> vertices;     // x y z pad per vertex (the reference's Vertex layout)
    std::vector<uint32_t> indices;   // v0 v1 v2 per triangle
    size_t numTris = 0, numVerts = 0;
};
struct ShimScene {
    std::vector<ShimMesh> meshes;
};

// Returns hit distance or -1 for a miss; u, v are the barycentrics of v1, v2.
inline double HitTriangle(const RTCRay &ray, const float *p0, const float *p1, const float *p2,
                          double &u, double &v) {
    const double o[3] = {ray.org[0], ray.org[1], ray.org[2]};
    const double d[3] = {ray.dir[0], ray.dir[1], ray.dir[2]};
    double e1[3], e2[3], s[3];
    for (int k = 0; k < 3; k++) {
        e1[k] = double(p1[k]) - p0[k];
        e2[k] = double(p2[k]) - p0[k];
        s[k] = o[k] - p0[k];
    }
    const double pv[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2],
                          d[0] * e2[1] - d[1] * e2[0]};
    const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
    if (det == 0.0) return -1.0;
    const double inv = 1.0 / det;
    u = (s[0] * pv[0] + s[1] * pv[1] + s[2] * pv[2]) * inv;
    if (u < 0.0 || u > 1.0) return -1.0;
    const double q[3] = {s[1] * e1[2] - s[2] * e1[1], s[2] * e1[0] - s[0] * e1[2],
                         s[0] * e1[1] - s[1] * e1[0]};
    v = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * inv;
    if (v < 0.0 || u + v > 1.0) return -1.0;
    return (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * inv;
}

template <bool anyHit>
void Trace(RTCScene scene, RTCRay &ray) {
    const ShimScene *s = reinterpret_cast<const ShimScene *>(scene);
    double best = ray.tfar;
    for (size_t g = 0; g < s->meshes.size(); g++) {
        const ShimMesh &m = s->meshes[g];
        for (size_t t = 0; t < m.numTris; t++) {
            const uint32_t *idx = &m.indices[3 * t];
            double u, v;
            const double hit = HitTriangle(ray, &m.vertices[4 * idx[0]], &m.vertices[4 * idx[1]],
                                           &m.vertices[4 * idx[2]], u, v);
            if (hit > ray.tnear && hit <= best) {
                if (anyHit) {
                    ray.geomID = 0;  // Embree reports occlusion by zeroing geomID
                    return;
                }
                best = hit;
                ray.tfar = float(hit);
                ray.u = float(u);
                ray.v = float(v);
                ray.geomID = unsigned(g);
                ray.primID = unsigned(t);
            }
        }
    }
}
}  // namespace

RTCDevice rtcNewDevice(const char *) { return reinterpret_cast<RTCDevice>(new int(0)); }
void rtcDeleteDevice(RTCDevice device) { delete reinterpret_cast<int *>(device); }
RTCScene rtcDeviceNewScene(RTCDevice, RTCSceneFlags, RTCAlgorithmFlags) {
    return reinterpret_cast<RTCScene>(new ShimScene());
}
void rtcDeleteScene(RTCScene scene) { delete reinterpret_cast<ShimScene *>(scene); }
unsigned rtcNewTriangleMesh(RTCScene scene, RTCGeometryFlags, size_t numTriangles,
                            size_t numVertices, size_t) {
    ShimScene *s = reinterpret_cast<ShimScene *>(scene);
    s->meshes.emplace_back();
    ShimMesh &m = s->meshes.back();
    m.numTris = numTriangles;
    m.numVerts = numVertices;
    m.vertices.resize(4 * numVertices);
    m.indices.resize(3 * numTriangles);
    return unsigned(s->meshes.size() - 1);
}
void *rtcMapBuffer(RTCScene scene, unsigned geomID, RTCBufferType type) {
    ShimMesh &m = reinterpret_cast<ShimScene *>(scene)->meshes[geomID];
    if (type == RTC_INDEX_BUFFER) return m.indices.data();
    return m.vertices.data();  // RTC_VERTEX_BUFFER / RTC_VERTEX_BUFFER0 (static scenes only)
}
void rtcUnmapBuffer(RTCScene, unsigned, RTCBufferType) {}
void rtcCommit(RTCScene) {}
void rtcIntersect(RTCScene scene, RTCRay &ray) { Trace<false>(scene, ray); }
void rtcOccluded(RTCScene scene, RTCRay &ray) { Trace<true>(scene, ray); }
