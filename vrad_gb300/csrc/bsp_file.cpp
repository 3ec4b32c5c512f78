// bsp_file.cpp -- the lumps of a compiled Source map (BSP versions 19-21)
// that the brush ingest reads, decoded from the file's bytes into the arrays
// of vrg_bsp_world.  The reference reads the same lumps through galaco/bsp
// (cmd/tasks/loadbsp/main.go:31-40, cache/lumps.go), which is not part of the
// project; the record layouts below are those of the public Source BSP
// format, little-endian:
//   header: "VBSP", int version, 64 x {int fileofs, int filelen, int
//           version, char fourCC[4]} (fourCC != 0: compressed), int revision
//   1  planes      20 B  {float normal[3], float dist, int type}
//   3  vertexes    12 B  {float x, y, z}
//   5  nodes       32 B  {int planenum, int children[2], short mins[3],
//                         short maxs[3], u16 firstface, u16 numfaces,
//                         short area, short pad}
//   6  texinfo     72 B  {float texvecs[2][4], float lightmapvecs[2][4],
//                         int flags, int texdata}
//   7  faces       56 B  {u16 planenum, u8 side, u8 onnode, int firstedge,
//                         short numedges, short texinfo, short dispinfo,
//                         short fogvolume, u8 styles[4], int lightofs,
//                         float area, int lmmins[2], int lmsize[2],
//                         int origface, u16 numprims, u16 firstprim,
//                         u32 smoothing}
//   10 leafs       32 B (lump version 1) or 56 B (version 0, with the
//                  ambient cube): {int contents, short cluster, short
//                  area_flags, short mins[3], short maxs[3], u16
//                  firstleafface, u16 numleaffaces, u16 firstleafbrush,
//                  u16 numleafbrushes, short waterdata, ...}
//   12 edges        4 B  {u16 v[2]}
//   13 surfedges    4 B  int
//   14 models      48 B  {float mins[3], maxs[3], origin[3], int headnode,
//                         int firstface, int numfaces}
//   17 leafbrushes  2 B  u16
//   18 brushes     12 B  {int firstside, int numsides, int contents}
//   19 brushsides   8 B  {u16 planenum, short texinfo, short dispinfo,
//                         u8 bevel, u8 thin}
//   58 faces (HDR)  56 B  as lump 7
// Bytes are read with memcpy and assembled little-endian, so the decode is
// the same on any host.
#include <cstring>
#include <new>
#include <vector>

#include "vrg_internal.h"

struct vrg_bsp {
    int32_t version = 0;
    bool hdr = false;  // the world's faces from the HDR face lump
    std::vector<float> planes, vertexes;
    std::vector<int32_t> node_children, leaf_brush_ranges, leaf_brushes, brushes, brush_sides,
        texinfo_flags, edges, surf_edges, faces, faces_hdr;
    std::vector<float> lightmap_vecs;  // 8 per texinfo
    int32_t headnode = 0, first_face = 0, num_model_faces = 0;
};

namespace {

enum {
    kPlanes = 1, kVertexes = 3, kNodes = 5, kTexinfo = 6, kFaces = 7, kLeafs = 10, kEdges = 12,
    kSurfEdges = 13, kModels = 14, kLeafBrushes = 17, kBrushes = 18, kBrushSides = 19, kFacesHdr = 58,
    kNumLumps = 64
};
constexpr size_t kHeaderBytes = 8 + 16 * kNumLumps + 4;

uint32_t rd32(const uint8_t *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
int32_t ri32(const uint8_t *p) { return (int32_t)rd32(p); }
uint16_t ru16(const uint8_t *p) { return (uint16_t)(p[0] | (p[1] << 8)); }
int16_t ri16(const uint8_t *p) { return (int16_t)ru16(p); }
float rf32(const uint8_t *p) {
    const uint32_t u = rd32(p);
    float f;
    memcpy(&f, &u, 4);
    return f;
}

struct Lump {
    const uint8_t *p = nullptr;
    size_t bytes = 0;
    int32_t version = 0;
};

}  // namespace

using namespace vrg;

extern "C" {

int vrg_bsp_open(const uint8_t *data, size_t size, vrg_bsp **out) {
    if (!out) return VRG_ERR_INVALID;
    *out = nullptr;
    if (!data || size < kHeaderBytes || memcmp(data, "VBSP", 4) != 0) return VRG_ERR_INVALID;
    const int32_t version = ri32(data + 4);
    if (version < 19 || version > 21) return VRG_ERR_UNSUPPORTED;
    Lump L[kNumLumps];
    for (int i = 0; i < kNumLumps; i++) {
        const uint8_t *e = data + 8 + 16 * i;
        const int64_t ofs = ri32(e), len = ri32(e + 4);
        if (ofs < 0 || len < 0 || (uint64_t)(ofs + len) > size) return VRG_ERR_INVALID;
        L[i] = Lump{data + ofs, (size_t)len, ri32(e + 8)};
        const bool used = i == kPlanes || i == kVertexes || i == kNodes || i == kTexinfo || i == kFaces ||
                          i == kLeafs || i == kEdges || i == kSurfEdges || i == kModels ||
                          i == kLeafBrushes || i == kBrushes || i == kBrushSides || i == kFacesHdr;
        if (used && len > 0 && rd32(e + 12) != 0) return VRG_ERR_UNSUPPORTED;  // compressed lump
    }
    const size_t leaf_bytes = L[kLeafs].version == 0 ? 56 : 32;
    const struct {
        int lump;
        size_t rec;
    } sizes[] = {{kPlanes, 20}, {kVertexes, 12}, {kNodes, 32}, {kTexinfo, 72}, {kFaces, 56}, {kFacesHdr, 56},
                 {kLeafs, leaf_bytes}, {kEdges, 4}, {kSurfEdges, 4}, {kModels, 48}, {kLeafBrushes, 2},
                 {kBrushes, 12}, {kBrushSides, 8}};
    for (const auto &s : sizes)
        if (L[s.lump].bytes % s.rec != 0 || L[s.lump].bytes / s.rec > (size_t)INT32_MAX) return VRG_ERR_INVALID;
    vrg_bsp *b = new (std::nothrow) vrg_bsp();
    if (!b) return VRG_ERR_NOMEM;
    b->version = version;
    try {
        for (size_t i = 0; i < L[kPlanes].bytes / 20; i++)
            for (int k = 0; k < 4; k++) b->planes.push_back(rf32(L[kPlanes].p + 20 * i + 4 * k));
        for (size_t i = 0; i < L[kVertexes].bytes / 4; i++) b->vertexes.push_back(rf32(L[kVertexes].p + 4 * i));
        for (size_t i = 0; i < L[kNodes].bytes / 32; i++) {
            b->node_children.push_back(ri32(L[kNodes].p + 32 * i + 4));
            b->node_children.push_back(ri32(L[kNodes].p + 32 * i + 8));
        }
        for (size_t i = 0; i < L[kTexinfo].bytes / 72; i++) {
            const uint8_t *t = L[kTexinfo].p + 72 * i;
            for (int k = 0; k < 8; k++) b->lightmap_vecs.push_back(rf32(t + 32 + 4 * k));
            b->texinfo_flags.push_back(ri32(t + 64));
        }
        for (int lump : {kFaces, kFacesHdr}) {
            std::vector<int32_t> &dst = lump == kFaces ? b->faces : b->faces_hdr;
            for (size_t i = 0; i < L[lump].bytes / 56; i++) {
                const uint8_t *f = L[lump].p + 56 * i;
                dst.push_back(ri32(f + 4));   // firstedge
                dst.push_back(ri16(f + 8));   // numedges
                dst.push_back(ri16(f + 10));  // texinfo
            }
        }
        for (size_t i = 0; i < L[kLeafs].bytes / leaf_bytes; i++) {
            const uint8_t *l = L[kLeafs].p + leaf_bytes * i;
            b->leaf_brush_ranges.push_back(ru16(l + 24));
            b->leaf_brush_ranges.push_back(ru16(l + 26));
        }
        for (size_t i = 0; i < L[kEdges].bytes / 2; i++) b->edges.push_back(ru16(L[kEdges].p + 2 * i));
        for (size_t i = 0; i < L[kSurfEdges].bytes / 4; i++) b->surf_edges.push_back(ri32(L[kSurfEdges].p + 4 * i));
        for (size_t i = 0; i < L[kLeafBrushes].bytes / 2; i++)
            b->leaf_brushes.push_back(ru16(L[kLeafBrushes].p + 2 * i));
        for (size_t i = 0; i < L[kBrushes].bytes / 4; i++) b->brushes.push_back(ri32(L[kBrushes].p + 4 * i));
        for (size_t i = 0; i < L[kBrushSides].bytes / 8; i++) {
            const uint8_t *s = L[kBrushSides].p + 8 * i;
            b->brush_sides.push_back(ru16(s));
            b->brush_sides.push_back(ri16(s + 2));
            b->brush_sides.push_back(ri16(s + 4));
            b->brush_sides.push_back(s[6]);
        }
    } catch (const std::bad_alloc &) {
        delete b;
        return VRG_ERR_NOMEM;
    }
    if (L[kModels].bytes >= 48) {  // model 0: the world
        const uint8_t *m = L[kModels].p;
        b->headnode = ri32(m + 36);
        b->first_face = ri32(m + 40);
        b->num_model_faces = ri32(m + 44);
    }
    *out = b;
    return VRG_OK;
}

void vrg_bsp_close(vrg_bsp *bsp) { delete bsp; }

int vrg_bsp_get_world(const vrg_bsp *b, vrg_bsp_world *w) {
    if (!b || !w) return VRG_ERR_INVALID;
    auto p = [](const auto &v) { return v.empty() ? nullptr : v.data(); };
    w->planes = p(b->planes);
    w->num_planes = (int32_t)(b->planes.size() / 4);
    w->node_children = p(b->node_children);
    w->num_nodes = (int32_t)(b->node_children.size() / 2);
    w->leaf_brush_ranges = p(b->leaf_brush_ranges);
    w->num_leafs = (int32_t)(b->leaf_brush_ranges.size() / 2);
    w->leaf_brushes = p(b->leaf_brushes);
    w->num_leaf_brushes = (int32_t)b->leaf_brushes.size();
    w->brushes = p(b->brushes);
    w->num_brushes = (int32_t)(b->brushes.size() / 3);
    w->brush_sides = p(b->brush_sides);
    w->num_brush_sides = (int32_t)(b->brush_sides.size() / 4);
    w->texinfo_flags = p(b->texinfo_flags);
    w->num_texinfo = (int32_t)b->texinfo_flags.size();
    w->vertexes = p(b->vertexes);
    w->num_vertexes = (int32_t)(b->vertexes.size() / 3);
    w->edges = p(b->edges);
    w->num_edges = (int32_t)(b->edges.size() / 2);
    w->surf_edges = p(b->surf_edges);
    w->num_surf_edges = (int32_t)b->surf_edges.size();
    const std::vector<int32_t> &faces = b->hdr ? b->faces_hdr : b->faces;
    w->faces = p(faces);
    w->num_faces = (int32_t)(faces.size() / 3);
    w->headnode = b->headnode;
    w->first_face = b->first_face;
    w->num_model_faces = b->num_model_faces;
    return VRG_OK;
}

int vrg_bsp_use_hdr_faces(vrg_bsp *b, int32_t hdr) {
    if (!b) return VRG_ERR_INVALID;
    b->hdr = hdr != 0;
    return VRG_OK;
}

int vrg_bsp_info(const vrg_bsp *b, int32_t *version, int32_t *num_texinfo, const float **lightmap_vecs) {
    if (!b) return VRG_ERR_INVALID;
    if (version) *version = b->version;
    if (num_texinfo) *num_texinfo = (int32_t)b->texinfo_flags.size();
    if (lightmap_vecs) *lightmap_vecs = b->lightmap_vecs.empty() ? nullptr : b->lightmap_vecs.data();
    return VRG_OK;
}

}  // extern "C"
