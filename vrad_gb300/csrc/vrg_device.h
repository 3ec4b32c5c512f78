// vrg_device.h -- plain-old-data layouts shared by host code and kernels.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
#include <vector_types.h>
#endif

namespace vrg {

// One triangle in intersection form, as three 16-byte words so a kernel
// fetches it with three vector loads:
//   w0 = (Nx, Ny, Nz, D)         plane (TriIntersectData.FlNx..FlD)
//   w1 = (e0, e1, e2, e3)        ProjectedEdgeEquations[0..3]
//   w2 = (e4, e5, id, idx_drop)  ProjectedEdgeEquations[4..5], NTriangleID,
//                                (triangle index << 2) | dropped axis
// The coordinates kept for the edge test are (drop+1)%3 and (drop+2)%3
// (NCoordSelect0/1 of raytracer/cache/optimisedtriangle.go:63-67).
struct alignas(16) TriRecord {
    float nx, ny, nz, d;
    float e0, e1, e2, e3;
    float e4, e5;
    int32_t id;
    uint32_t idx_drop;
};
static_assert(sizeof(TriRecord) == 48, "TriRecord must be 48 bytes");

// Wall slots: per face of the scene box (2 * axis + 1 for the max side), up
// to kWallSlots opaque triangles lying in that face, as extra leaf records.
constexpr int kWallSlots = 4;

struct SceneGeom {
    float bmin[3], bmax[3];  // root bounds (CalculateTriangleListBounds)
    float smin[3], smax[3];  // bounds of TRACE_ID_SKY triangles
    float scale;             // largest |coordinate| of any vertex
    int32_t has_sky;
    int64_t ntris;
    uint32_t wall_count;     // 3 bits per box face: its wall slots in use
    uint32_t wall_base;      // leaf-record index of face 0's first wall slot
};

// Device view of a resident scene.  The triangle records of the leaves are
// split in two arrays indexed by TriangleIndexList position: the plane
// (Nx, Ny, Nz, D), which the test reads first and which rejects most
// triangles, and the edge part (e0..e3), (e4, e5, id, index<<2 | drop).
struct DevScene {
    const uint2 *nodes;         // (children, split bits) per kd node
    const float4 *leaf_planes;  // 1 float4 per TriangleIndexList entry
    const float4 *leaf_edges;   // 2 float4 per TriangleIndexList entry
    const int32_t *tri_ids;     // NTriangleID per triangle index
    const uint2 *top;           // top levels of the tree in breadth-first order (see kTopRef)
    uint32_t ntop;              // entries of `top` (0: none)
    SceneGeom g;
};

// The top table holds the first kTopNodes nodes of a breadth-first walk from
// the root, children pairs kept adjacent.  A child word there whose index
// has kTopRef set points into the table instead of the node array, so a
// walk that stages the table in shared memory reads the top levels there.
constexpr int kTopNodes = 512;
constexpr uint32_t kTopRef = 1u << 27;

// Children word of an inner node on the device: axis (bits 0-1), index of
// the left child with kTopRef (bits 2-29), and whether the left (bit 31) or
// the right (bit 30) child is a leaf without triangles, so that the walk
// never fetches or stacks such a child.  Leaf words are 3 | first record << 2.
constexpr uint32_t kLeftEmpty = 1u << 31;
constexpr uint32_t kRightEmpty = 1u << 30;
constexpr uint32_t kChildIndexMask = (1u << 28) - 1u;  // after >> 2

// Lightmapped face, 80 bytes.
struct alignas(16) FaceRec {
    float4 corner;  // xyz, w = luxscale
    float4 u;       // xyz
    float4 v;       // xyz
    float4 normal;  // xyz
    int32_t nu, nv;
    int32_t pad0, pad1;
};
static_assert(sizeof(FaceRec) == 80, "FaceRec must be 80 bytes");

// Internal node of a face's patch tree, or a leaf (axis < 0).
struct alignas(16) PatchNode {
    int32_t child1;  // coordinate >= dist goes here (ClipWindingEpsilon front)
    int32_t child2;
    int32_t axis;    // split axis, -1 for a leaf
    union {
        float dist;
        int32_t leaf;  // dense leaf index when axis < 0
    };
};

// Per leaf patch, what the transfer and bounce kernels read.
struct alignas(16) LeafInfo {
    float4 center;  // xyz, w = area
    float4 refl;    // xyz reflectivity, w = face index (as float bits)
    float4 base;    // xyz baselight
};

constexpr int kStackMax = 32;
// common/constants/constants.go:19 MAX_TRACE_LENGTH = 1.732050807569 * 32768
constexpr float kMaxTraceLength = (float)(1.732050807569 * 32768.0);
// sample points and transfer origins sit this far off their surface
constexpr float kSampleOffset = 0.125f;
constexpr int kNumAnorms = 162;

}  // namespace vrg
