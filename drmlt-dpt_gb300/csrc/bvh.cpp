// Host SAH BVH builder: binned SAH (16 bins per axis), leaves of at most 4
// triangles, emitted as binary nodes that hold both children's boxes so a
// traversal step tests two boxes with one 64-byte load. Replaces the Embree
// scene build of src/scene.cpp:42-53.
#include "bvh.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

namespace drmlt {
namespace {

struct Box {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const Box &b) {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    void grow(const float *p) {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    float area() const {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (dx < 0.0f) return 0.0f;
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct Prim {
    Box box;
    float c[3];
    int id;
};

struct Builder {
    std::vector<Prim> prims;
    std::vector<BvhNode> nodes;
    static constexpr int kLeaf = 4;
    static constexpr int kBins = 16;

    // Returns a child reference: (index, count) where count > 0 denotes a leaf.
    void build(int begin, int end, const Box &box, int &ref, int &count) {
        const int n = end - begin;
        if (n <= kLeaf) {
            ref = begin;
            count = n;
            return;
        }
        Box cbox;
        for (int i = begin; i < end; i++) cbox.grow(prims[i].c);
        int bestAxis = -1, bestSplit = -1;
        float bestCost = FLT_MAX;
        for (int axis = 0; axis < 3; axis++) {
            const float ext = cbox.hi[axis] - cbox.lo[axis];
            if (ext <= 0.0f) continue;
            Box bins[kBins];
            int cnt[kBins] = {0};
            for (int i = begin; i < end; i++) {
                int b = int(kBins * (prims[i].c[axis] - cbox.lo[axis]) / ext);
                b = std::min(std::max(b, 0), kBins - 1);
                bins[b].grow(prims[i].box);
                cnt[b]++;
            }
            Box left[kBins];
            int lc[kBins];
            Box acc;
            int accN = 0;
            for (int b = 0; b < kBins; b++) {
                acc.grow(bins[b]);
                accN += cnt[b];
                left[b] = acc;
                lc[b] = accN;
            }
            Box racc;
            int raccN = 0;
            for (int b = kBins - 1; b > 0; b--) {
                racc.grow(bins[b]);
                raccN += cnt[b];
                if (lc[b - 1] == 0 || raccN == 0) continue;
                const float cost = left[b - 1].area() * lc[b - 1] + racc.area() * raccN;
                if (cost < bestCost) {
                    bestCost = cost;
                    bestAxis = axis;
                    bestSplit = b;
                }
            }
        }
        int mid;
        if (bestAxis < 0) {
            mid = begin + n / 2;  // all centroids coincide: split by count
        } else {
            const float ext = cbox.hi[bestAxis] - cbox.lo[bestAxis];
            auto it = std::partition(prims.begin() + begin, prims.begin() + end, [&](const Prim &p) {
                int b = int(kBins * (p.c[bestAxis] - cbox.lo[bestAxis]) / ext);
                b = std::min(std::max(b, 0), kBins - 1);
                return b < bestSplit;
            });
            mid = int(it - prims.begin());
            if (mid == begin || mid == end) mid = begin + n / 2;
        }
        Box lb, rb;
        for (int i = begin; i < mid; i++) lb.grow(prims[i].box);
        for (int i = mid; i < end; i++) rb.grow(prims[i].box);
        const int self = int(nodes.size());
        nodes.emplace_back();
        int r0, c0, r1, c1;
        build(begin, mid, lb, r0, c0);
        build(mid, end, rb, r1, c1);
        BvhNode &nd = nodes[self];
        nd.lo0 = make_float4(lb.lo[0], lb.lo[1], lb.lo[2], lb.hi[0]);
        nd.hi0 = make_float4(lb.hi[1], lb.hi[2], rb.lo[0], rb.lo[1]);
        nd.b1 = make_float4(rb.lo[2], rb.hi[0], rb.hi[1], rb.hi[2]);
        nd.link = make_int4(r0, r1, c0, c1);
        ref = self;
        count = 0;
    }
};

}  // namespace

void BuildBvh(const float *triP, const int *triShape, int numTris, std::vector<BvhNode> &nodes,
              std::vector<Tri> &tris) {
    Builder b;
    b.prims.resize(numTris);
    Box root;
    for (int t = 0; t < numTris; t++) {
        const float *P = triP + 9 * t;
        Prim &p = b.prims[t];
        float v[3][3];
        for (int k = 0; k < 3; k++) {
            v[0][k] = P[k];
            v[1][k] = P[k] + P[3 + k];
            v[2][k] = P[k] + P[6 + k];
        }
        for (int j = 0; j < 3; j++) p.box.grow(v[j]);
        // pad flat boxes so that slab tests never see a zero-extent axis
        for (int k = 0; k < 3; k++) {
            const float pad = 1e-6f * std::max(1.0f, std::fabs(p.box.hi[k]));
            p.box.lo[k] -= pad;
            p.box.hi[k] += pad;
        }
        for (int k = 0; k < 3; k++) p.c[k] = 0.5f * (p.box.lo[k] + p.box.hi[k]);
        p.id = t;
        root.grow(p.box);
    }
    b.nodes.reserve(2 * numTris / Builder::kLeaf + 2);
    int ref, count;
    if (numTris <= Builder::kLeaf) {
        // single leaf under a root node with an empty second child
        BvhNode nd;
        nd.lo0 = make_float4(root.lo[0], root.lo[1], root.lo[2], root.hi[0]);
        nd.hi0 = make_float4(root.hi[1], root.hi[2], 1.0f, 1.0f);
        nd.b1 = make_float4(1.0f, -1.0f, -1.0f, -1.0f);  // inverted box: never hit
        nd.link = make_int4(0, -1, numTris, 0);
        b.nodes.push_back(nd);
    } else {
        b.build(0, numTris, root, ref, count);
    }
    nodes = b.nodes;
    tris.resize(numTris);
    for (int i = 0; i < numTris; i++) {
        const int t = b.prims[i].id;
        const float *P = triP + 9 * t;
        Tri &o = tris[i];
        int gid = t, sid = triShape[t];
        float fg, fs;
        std::memcpy(&fg, &gid, 4);
        std::memcpy(&fs, &sid, 4);
        o.p0 = make_float4(P[0], P[1], P[2], fg);
        o.e1 = make_float4(P[3], P[4], P[5], fs);
        o.e2 = make_float4(P[6], P[7], P[8], 0.0f);
    }
}

}  // namespace drmlt
