// vbx.cpp -- GVDB .vbx files (gvdb-voxel-src/GVDB_FILESPEC.txt; the reader follows the field
// order of VolumeGVDB::LoadVBX, gvdb_volume_gvdb.cpp:532-700, and the node/id layouts that
// Scene::addGVDBVolume repacks, Scene.cpp:2898-3058).
//
// Reading: the grid's tree is walked from its root through the child lists, as the renderer's
// lookups do; every reachable leaf (an 8^3 brick) is copied out of the atlas at its value
// coordinate into a dense mip-0 grid over the grid's effective voxel box (x.12 files) or the
// leaves' box, and the volume (normal and conservative mips, brick bounds) is built from it by
// build_volume, or by build_signed_grid for signed data (velocity components).
//
// Writing: mip 0 of a volume as one float grid in the three-level layout the renderer's
// unrolled lookup expects (log2 dims 3, 4, 5), atlas layout with a one-voxel apron, no
// bitmasks, format version 1.12 (grid transform: scale = voxel size, translation = world_min;
// effective voxel box [0, res)^3).
//
// Supported on read: versions 1.0 - 2.x (bitmasks skipped), float data with one component, no
// compression, GVDB topology, atlas layout, 8^3 leaves, no rotation, uniform scale.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "vr_volume.h"

namespace vr {
namespace {

constexpr uint64_t kIdUndef = 0xFFFFFFFFFFFFFFFFull;
constexpr int kNodeBytes = 64;          // nvdb::Node (gvdb_node.h:40-53)

// pool ids: group in bits 0-7, level in bits 8-15, index in bits 16-47
inline uint64_t make_id(int lev, uint64_t index) { return ((uint64_t)lev << 8) | (index << 16); }
inline int id_level(uint64_t id) { return (int)((id >> 8) & 0xFF); }
inline int64_t id_index(uint64_t id) { return (int64_t)((id >> 16) & 0xFFFFFFFFull); }

struct Reader {
    const unsigned char* p;
    size_t n, off = 0;
    bool ok = true;
    template <class T>
    T get() {
        T v{};
        if (off + sizeof(T) > n) { ok = false; return v; }
        memcpy(&v, p + off, sizeof(T));
        off += sizeof(T);
        return v;
    }
    void skip(size_t k) { if (off + k > n) ok = false; else off += k; }
};

struct Node {
    int pos[3], value[3];
    uint64_t childList;
};

inline Node node_at(const std::vector<unsigned char>& pool, int width, int64_t i) {
    Node d;
    const unsigned char* q = pool.data() + (size_t)i * width;
    memcpy(d.pos, q + 4, 12);
    memcpy(d.value, q + 16, 12);
    memcpy(&d.childList, q + 48, 8);
    return d;
}

struct Writer {
    std::vector<unsigned char> b;
    template <class T>
    void put(const T& v) {
        const unsigned char* q = reinterpret_cast<const unsigned char*>(&v);
        b.insert(b.end(), q, q + sizeof(T));
    }
    void bytes(const void* q, size_t k) { b.insert(b.end(), (const unsigned char*)q, (const unsigned char*)q + k); }
};

}  // namespace

int read_vbx(const std::vector<unsigned char>& file, int numMips, bool fp16, bool signedValues, Volume& vol, std::string& err) {
    Reader r{file.data(), file.size()};
    const int major = r.get<uint8_t>(), minor = r.get<uint8_t>();
    float pretrans[3] = {0, 0, 0}, angs[3] = {0, 0, 0}, scale[3] = {1, 1, 1}, trans[3] = {0, 0, 0};
    if ((major == 1 && minor >= 11) || major > 1) {
        for (float& v : pretrans) v = r.get<float>();
        for (float& v : angs) v = r.get<float>();
        for (float& v : scale) v = r.get<float>();
        for (float& v : trans) v = r.get<float>();
    }
    // version x.12 (the reference's GVDB): VDB transforms, the effective voxel box, value range
    int effMin[3] = {0, 0, 0}, effMax[3] = {0, 0, 0};
    bool hasBox = false;
    if (minor == 12) {
        r.skip(16 * 4 * 2);
        for (int& v : effMin) v = r.get<int32_t>();
        for (int& v : effMax) v = r.get<int32_t>();
        r.skip(8);
        hasBox = effMax[0] > effMin[0] && effMax[1] > effMin[1] && effMax[2] > effMin[2];
    }
    const int numGrids = r.get<int32_t>();
    int readMasks = 0;
    if (major >= 2) readMasks = r.get<uint8_t>();
    else if (major == 1 && minor == 0) readMasks = 1;
    if (!r.ok || numGrids < 1 || numGrids > 4096) { err = "not a VBX file (header)"; return 1; }
    std::vector<uint64_t> gridOffs(numGrids);
    for (auto& g : gridOffs) g = r.get<uint64_t>();
    // grid 0
    char name[256];
    for (char& ch : name) ch = (char)r.get<uint8_t>();
    const char dtype = (char)r.get<uint8_t>();
    const int comps = r.get<uint8_t>();
    const int compress = r.get<uint8_t>();
    r.skip(12);                                             // voxel size (deprecated)
    const int leafCnt = r.get<int32_t>();
    int leafDim[3];
    for (int& v : leafDim) v = r.get<int32_t>();
    const int apron = r.get<int32_t>();
    const int numChan = r.get<int32_t>();
    r.get<uint64_t>();                                      // atlas size (all channels)
    const int topo = r.get<uint8_t>();
    r.get<int32_t>();                                       // topology reuse grid
    const int layout = r.get<uint8_t>();
    int axisCnt[3], axisRes[3];
    for (int& v : axisCnt) v = r.get<int32_t>();
    for (int& v : axisRes) v = r.get<int32_t>();
    const int levels = r.get<int32_t>();
    const uint64_t root = r.get<uint64_t>();
    if (!r.ok) { err = "truncated VBX grid header"; return 1; }
    if (dtype != 'f' || comps != 1) { err = "only float grids with one component are supported"; return 1; }
    if (compress != 0) { err = "compressed VBX grids are not supported"; return 1; }
    if (topo != 2 || layout != 0) { err = "only GVDB topology with atlas layout is supported"; return 1; }
    if (leafDim[0] != 8 || leafDim[1] != 8 || leafDim[2] != 8 || apron < 0 || apron > 4) { err = "leaves must be 8^3 bricks"; return 1; }
    if (levels < 1 || levels > 10 || numChan < 1 || leafCnt < 0) { err = "bad VBX topology header"; return 1; }
    if (angs[0] != 0.f || angs[1] != 0.f || angs[2] != 0.f || scale[0] != scale[1] || scale[1] != scale[2] || !(scale[0] > 0.f)) {
        err = "rotated or anisotropic VBX grids are not supported"; return 1;
    }
    std::vector<int> ld(levels), res(levels), cnt0(levels), w0(levels), cnt1(levels), w1(levels);
    for (int l = 0; l < levels; ++l) {
        ld[l] = r.get<int32_t>();
        res[l] = r.get<int32_t>();
        r.skip(12);                                         // range
        cnt0[l] = r.get<int32_t>();
        w0[l] = r.get<int32_t>();
        cnt1[l] = r.get<int32_t>();
        w1[l] = r.get<int32_t>();
        if (!r.ok || cnt0[l] < 0 || cnt1[l] < 0 || w0[l] < kNodeBytes || w1[l] < 0 || ld[l] < 1 || ld[l] > 12 || res[l] != (1 << ld[l])) {
            err = "bad VBX level header"; return 1;
        }
        if (l > 0 && cnt1[l] > 0 && w1[l] < (int64_t)res[l] * res[l] * res[l] * 8) { err = "VBX child list narrower than the level's resolution"; return 1; }
    }
    if (ld[0] != 3) { err = "leaves must be 8^3 bricks"; return 1; }
    (void)readMasks;                                        // bitmasks live inside the node rows (width0 > 64) and are skipped
    std::vector<std::vector<unsigned char>> pool0(levels), pool1(levels);
    for (int l = 0; l < levels; ++l) {
        const size_t k = (size_t)cnt0[l] * w0[l];
        if (r.off + k > r.n) { err = "truncated VBX node pool"; return 1; }
        pool0[l].assign(file.begin() + r.off, file.begin() + r.off + k);
        r.off += k;
    }
    for (int l = 0; l < levels; ++l) {
        const size_t k = (size_t)cnt1[l] * w1[l];
        if (r.off + k > r.n) { err = "truncated VBX child pool"; return 1; }
        pool1[l].assign(file.begin() + r.off, file.begin() + r.off + k);
        r.off += k;
    }
    r.get<int32_t>();                                       // channel 0 type
    const int stride = r.get<int32_t>();
    if (!r.ok || stride != 4) { err = "atlas channel 0 must hold 4-byte floats"; return 1; }
    const size_t atlasVox = (size_t)axisRes[0] * axisRes[1] * axisRes[2];
    if (axisRes[0] <= 0 || axisRes[1] <= 0 || axisRes[2] <= 0 || r.off + atlasVox * 4 > r.n) { err = "truncated VBX atlas"; return 1; }
    const size_t atlasOff = r.off;
    auto atlasAt = [&](int x, int y, int z) -> float {
        if (x < 0 || y < 0 || z < 0 || x >= axisRes[0] || y >= axisRes[1] || z >= axisRes[2]) return 0.f;
        float v;
        memcpy(&v, file.data() + atlasOff + (((size_t)z * axisRes[1] + y) * axisRes[0] + x) * 4, 4);
        return v;
    };
    // walk the tree from the root and collect the reachable leaves
    std::vector<Node> leaves;
    std::vector<uint64_t> stack{root};
    size_t visited = 0;
    while (!stack.empty()) {
        const uint64_t id = stack.back();
        stack.pop_back();
        if (id == kIdUndef) continue;
        const int lev = id_level(id);
        const int64_t idx = id_index(id);
        if (lev < 0 || lev >= levels || idx < 0 || idx >= cnt0[lev]) { err = "VBX node id out of range"; return 1; }
        if (++visited > (size_t)8 << 26) { err = "VBX tree too large"; return 1; }
        const Node nd = node_at(pool0[lev], w0[lev], idx);
        if (lev == 0) { leaves.push_back(nd); continue; }
        if (nd.childList == kIdUndef) continue;
        const int64_t row = id_index(nd.childList);
        if (row < 0 || row >= cnt1[lev]) { err = "VBX child list id out of range"; return 1; }
        const int64_t nch = (int64_t)res[lev] * res[lev] * res[lev];
        const unsigned char* q = pool1[lev].data() + (size_t)row * w1[lev];
        for (int64_t c = 0; c < nch; ++c) {
            uint64_t cid;
            memcpy(&cid, q + c * 8, 8);
            if (cid == kIdUndef || (uint32_t)cid == 0xFFFFFFFFu) continue;
            if (id_level(cid) != lev - 1) { err = "VBX child on the wrong level"; return 1; }
            stack.push_back(cid);
        }
    }
    // dense mip-0 grid over the effective voxel box (x.12 files), else over the leaves' box with
    // its corner aligned down to the mip pyramid's granularity, so coarse mips group the voxels
    // the same way; the side is padded to that granularity
    const int gran = 8 << (numMips - 1);
    int lo[3] = {0, 0, 0}, hi[3] = {gran, gran, gran};
    if (hasBox) {
        for (int a = 0; a < 3; ++a) { lo[a] = effMin[a]; hi[a] = effMax[a]; }
    } else if (!leaves.empty()) {
        for (int a = 0; a < 3; ++a) { lo[a] = leaves[0].pos[a]; hi[a] = leaves[0].pos[a] + 8; }
        for (const Node& l : leaves)
            for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], l.pos[a]); hi[a] = std::max(hi[a], l.pos[a] + 8); }
        for (int a = 0; a < 3; ++a) lo[a] = (int)std::floor((double)lo[a] / gran) * gran;
    }
    int R = 0;
    for (int a = 0; a < 3; ++a) R = std::max(R, hi[a] - lo[a]);
    R = (R + gran - 1) / gran * gran;
    if (R > 1024) { err = "VBX grid larger than 1024^3 voxels (dense reconstruction)"; return 1; }
    std::vector<float> dense((size_t)R * R * R, 0.f);
    for (const Node& l : leaves)
        for (int z = 0; z < 8; ++z)
            for (int y = 0; y < 8; ++y)
                for (int x = 0; x < 8; ++x) {
                    const int ix = l.pos[0] - lo[0] + x, iy = l.pos[1] - lo[1] + y, iz = l.pos[2] - lo[2] + z;
                    if (ix < 0 || iy < 0 || iz < 0 || ix >= R || iy >= R || iz >= R) continue;
                    float v = atlasAt(l.value[0] + x, l.value[1] + y, l.value[2] + z);
                    if (!(v == v) || std::isinf(v)) v = 0.f;
                    if (!signedValues && v < 0.f) v = 0.f;
                    dense[((size_t)iz * R + iy) * R + ix] = v;
                }
    // GVDB's transform: world = (index + pretranslation) * scale + translation
    float wmin[3];
    for (int a = 0; a < 3; ++a) wmin[a] = ((float)lo[a] + pretrans[a]) * scale[a] + trans[a];
    (void)name;
    const int rc = signedValues ? build_signed_grid(dense, R, wmin, scale[0], fp16, vol) : build_volume(dense, R, numMips, wmin, scale[0], fp16, vol);
    if (rc) { err = "volume build failed"; return 1; }
    return 0;
}

int write_vbx(const Volume& vol, std::vector<unsigned char>& out, std::string& err) {
    const GridSlot& s = vol.slots[0];
    if (!s.valid) { err = "volume has no mip 0"; return 1; }
    const int nb = s.num_bricks, nl1 = s.num_l1;
    // atlas: bricks on a near-cubic grid of (8 + 2) voxel cells
    int ac[3] = {1, 1, 1};
    while ((int64_t)ac[0] * ac[1] * ac[2] < std::max(1, nb)) {
        int a = (ac[0] <= ac[1] && ac[0] <= ac[2]) ? 0 : (ac[1] <= ac[2] ? 1 : 2);
        ac[a]++;
    }
    const int cell = 8 + 2;
    const int ar[3] = {ac[0] * cell, ac[1] * cell, ac[2] * cell};
    std::vector<float> atlas((size_t)ar[0] * ar[1] * ar[2], 0.f);
    auto brickVal = [&](int b, int i) { return s.brick_f32.empty() ? half_to_float(s.brick_f16[(size_t)b * 1000 + i]) : s.brick_f32[(size_t)b * 1000 + i]; };
    std::vector<int> bval((size_t)nb * 3);
    for (int b = 0; b < nb; ++b) {
        const int cz = b / (ac[0] * ac[1]), cy = (b / ac[0]) % ac[1], cx = b % ac[0];
        const int o[3] = {cx * cell, cy * cell, cz * cell};
        for (int z = 0; z < 10; ++z)
            for (int y = 0; y < 10; ++y)
                for (int x = 0; x < 10; ++x)
                    atlas[((size_t)(o[2] + z) * ar[1] + (o[1] + y)) * ar[0] + (o[0] + x)] = brickVal(b, (z * 10 + y) * 10 + x);
        for (int a = 0; a < 3; ++a) bval[(size_t)b * 3 + a] = o[a] + 1;
    }
    Writer w;
    w.put<uint8_t>(1); w.put<uint8_t>(12);
    const float zero3[3] = {0, 0, 0}, sc3[3] = {vol.voxel_size, vol.voxel_size, vol.voxel_size};
    w.bytes(zero3, 12); w.bytes(zero3, 12); w.bytes(sc3, 12); w.bytes(vol.world_min, 12);
    float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    w.bytes(ident, 64); w.bytes(ident, 64);                // VDB transform and inverse
    const int32_t boxMin[3] = {0, 0, 0}, boxMax[3] = {vol.res, vol.res, vol.res};
    w.bytes(boxMin, 12); w.bytes(boxMax, 12);
    const float vmin = 0.f, vmax = s.max_value;
    w.put<float>(vmin); w.put<float>(vmax);
    w.put<int32_t>(1);
    const size_t gridOffPos = w.b.size();
    w.put<uint64_t>(0);
    const uint64_t gridOff = w.b.size();
    memcpy(w.b.data() + gridOffPos, &gridOff, 8);
    char name[256] = {0};
    strncpy(name, "density", sizeof(name) - 1);
    w.bytes(name, 256);
    w.put<uint8_t>('f'); w.put<uint8_t>(1); w.put<uint8_t>(0);
    const float one3[3] = {1, 1, 1};
    w.bytes(one3, 12);
    w.put<int32_t>(nb);
    const int32_t leafDim[3] = {8, 8, 8};
    w.bytes(leafDim, 12);
    w.put<int32_t>(1);                                      // apron
    w.put<int32_t>(1);                                      // channels
    w.put<uint64_t>((uint64_t)atlas.size() * 4);
    w.put<uint8_t>(2); w.put<int32_t>(0); w.put<uint8_t>(0);
    w.bytes(ac, 12); w.bytes(ar, 12);
    w.put<int32_t>(3);
    w.put<uint64_t>(make_id(2, 0));
    const int lds[3] = {3, 4, 5};
    const int cnts0[3] = {nb, nl1, 1}, cnts1[3] = {0, nl1, 1};
    int range = 1;
    for (int l = 0; l < 3; ++l) {
        range *= 1 << lds[l];
        w.put<int32_t>(lds[l]); w.put<int32_t>(1 << lds[l]);
        const int32_t rg[3] = {range, range, range};
        w.bytes(rg, 12);
        w.put<int32_t>(cnts0[l]); w.put<int32_t>(kNodeBytes);
        w.put<int32_t>(cnts1[l]); w.put<int32_t>(l == 0 ? 0 : (1 << (3 * lds[l])) * 8);
    }
    auto node = [&](int lev, const int pos[3], const int val[3], uint64_t parent, uint64_t child) {
        unsigned char q[kNodeBytes] = {0};
        q[0] = (unsigned char)lev; q[1] = 1;
        memcpy(q + 4, pos, 12);
        memcpy(q + 16, val, 12);
        memcpy(q + 40, &parent, 8);
        memcpy(q + 48, &child, 8);
        const uint64_t mask = kIdUndef;
        memcpy(q + 56, &mask, 8);
        w.bytes(q, kNodeBytes);
    };
    // level 0 (bricks), level 1, level 2 (root)
    std::vector<int> parentOf(nb, 0);
    for (int l1 = 0; l1 < nl1; ++l1)
        for (int c = 0; c < 4096; ++c) {
            const int b = s.l1_child[(size_t)l1 * 4096 + c];
            if (b >= 0) parentOf[b] = l1;
        }
    for (int b = 0; b < nb; ++b) node(0, &s.brick_vmin[(size_t)b * 4], &bval[(size_t)b * 3], make_id(1, parentOf[b]), kIdUndef);
    const int zero[3] = {0, 0, 0};
    for (int l1 = 0; l1 < nl1; ++l1) node(1, &s.l1_vmin[(size_t)l1 * 4], zero, make_id(2, 0), make_id(1, l1));
    node(2, zero, zero, kIdUndef, make_id(2, 0));
    // child lists: level 1 (16^3 bricks each), level 2 (32^3 level-1 nodes)
    for (int l1 = 0; l1 < nl1; ++l1)
        for (int c = 0; c < 4096; ++c) {
            const int b = s.l1_child[(size_t)l1 * 4096 + c];
            w.put<uint64_t>(b >= 0 ? make_id(0, b) : kIdUndef);
        }
    for (int c = 0; c < 32768; ++c) {
        const int l1 = s.root_child[c];
        w.put<uint64_t>(l1 >= 0 ? make_id(1, l1) : kIdUndef);
    }
    w.put<int32_t>(3);                                      // channel type: float
    w.put<int32_t>(4);
    w.bytes(atlas.data(), atlas.size() * 4);
    out.swap(w.b);
    return 0;
}

}  // namespace vr
