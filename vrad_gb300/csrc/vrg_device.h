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

// Walls: per face of the scene box (2 * axis + 1 for the max side), the
// opaque triangles lying in that face as extra leaf records.  A face of at
// most kWallSlots of them keeps them in its slots (records wall_base +
// kWallSlots * face + i); a larger one gets a grid of at most kWallGridMax x
// kWallGridMax cells over the face, each listing at most kWallCellMax of the
// triangles that overlap it.  The cell table is one
// uint32 array: 6 face descriptors of kWallFaceWords words -- cell origin in
// the face's in-plane axes (a+1)%3, (a+2)%3 and inverse cell size (float
// bits), cells per axis, the table index of the face's cell starts -- then,
// per face with walls, gu * gv + 1 cell starts (table indices) followed by
// the cells' entries (leaf-record indices).  vrg_env_wall_slots reports the
// first kWallSlots triangles of each face.
constexpr int kWallSlots = 4;
constexpr int kWallGridMax = 32;
constexpr int kWallCellMax = 8;
constexpr int kWallFaceWords = 8;

struct SceneGeom {
    float bmin[3], bmax[3];  // root bounds (CalculateTriangleListBounds)
    float smin[3], smax[3];  // bounds of TRACE_ID_SKY triangles
    float scale;             // largest |coordinate| of any vertex
    int32_t has_sky;
    int64_t ntris;
    uint32_t wall_count;     // 3 bits per box face: its wall slots in use
    uint32_t wall_base;      // leaf-record index of face 0's first wall slot
    uint32_t wall_cell_mask; // bit f set: box face f has a wall-cell grid
};

// Device view of a resident scene.  The triangle records of the leaves are
// split in two arrays indexed by TriangleIndexList position: the plane
// (Nx, Ny, Nz, D), which the test reads first and which rejects most
// triangles, and the edge part (e0..e3), (e4, e5, id, index<<2 | drop).
// The entries are the tree's, then the walls' records; the wall-cell table
// follows the edge part in the same buffer (wall_table).  It has no pointer
// of its own: one more pointer in this kernel argument changed the
// direct-light kernel's register allocation and cost it 5 %.
struct DevScene {
    const uint2 *nodes;         // (children, split bits) per kd node
    const float4 *leaf_planes;  // 1 float4 per TriangleIndexList entry
    const float4 *leaf_edges;   // 2 float4 per TriangleIndexList entry
    const int32_t *tri_ids;     // NTriangleID per triangle index
    const uint2 *top;           // top levels of the tree in breadth-first order (see kTopRef)
    uint32_t ntop;              // entries of `top` (0: none)
    SceneGeom g;
};

// The wall-cell table (see kWallFaceWords), right after the edge part:
// leaf_edges - leaf_planes records, 2 float4 each.
__host__ __device__ inline const uint32_t *wall_table(const DevScene &s) {
    return reinterpret_cast<const uint32_t *>(s.leaf_edges + 2 * (s.leaf_edges - s.leaf_planes));
}

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
