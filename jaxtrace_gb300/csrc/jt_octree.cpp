// Host octree build over a tetrahedral mesh, following
// build_octree_mesh_optimized (fields/octree_fem_interpolator_optimized.py:41-215):
//   * element boxes = min/max of the four vertices, centroids = float32
//     ((p0+p1)+p2)+p3 then /4 (numpy mean over axis 0 of a (4,3) array);
//   * each tetrahedron goes to exactly one octant, chosen by its centroid
//     (>= the float32 node centre (min+max)/2 sets the octant bit);
//   * a node is a leaf when it holds <= max_elements_per_leaf elements or
//     sits at depth >= max_depth; nodes are numbered in DFS pre-order with
//     octants visited 0..7 and empty octants left as -1.
// The builder also emits the per-tetrahedron records the device lookup
// reads: a 32-byte box and a 64-byte geometry record (v0, v1-v0, v2-v0,
// v3-v0 rounded as float32, then the four vertex ids).
#include <stdint.h>
#include <string.h>

#include <new>
#include <vector>

#include "../../include/jaxtrace_gb300.h"
#include "jt_internal.h"

namespace {

struct Node {
    float mn[3], mx[3];
    int32_t children[8];
    bool leaf;
    int depth;
    int32_t elem_offset, elem_count;
};

struct Builder {
    const float* pts;
    const int32_t* conn;
    int32_t n_tets;
    int max_per_leaf, max_depth;
    std::vector<float> centroid;  // (n_tets,3)
    std::vector<Node> nodes;
    std::vector<int32_t> elems;   // leaf element lists, concatenated in node order
    int max_leaf_depth = 0;

    int32_t subdivide(const float* mn, const float* mx, std::vector<int32_t>& list, int depth) {
        const int32_t idx = (int32_t)nodes.size();
        Node nd;
        for (int a = 0; a < 3; ++a) { nd.mn[a] = mn[a]; nd.mx[a] = mx[a]; }
        for (int o = 0; o < 8; ++o) nd.children[o] = -1;
        nd.depth = depth;
        nd.leaf = ((int)list.size() <= max_per_leaf) || (depth >= max_depth);
        if (depth > max_leaf_depth) max_leaf_depth = depth;
        if (nd.leaf) {
            nd.elem_offset = (int32_t)elems.size();
            nd.elem_count = (int32_t)list.size();
            elems.insert(elems.end(), list.begin(), list.end());
            nodes.push_back(nd);
            return idx;
        }
        nd.elem_offset = (int32_t)elems.size();
        nd.elem_count = 0;
        float c[3];
        for (int a = 0; a < 3; ++a) {
            volatile float s = mn[a] + mx[a];  // float32 sum, then an exact halving
            c[a] = s / 2.0f;
        }
        std::vector<int32_t> oct[8];
        for (int32_t e : list) {
            const float* ce = &centroid[3 * (size_t)e];
            int o = 0;
            if (ce[0] >= c[0]) o += 1;
            if (ce[1] >= c[1]) o += 2;
            if (ce[2] >= c[2]) o += 4;
            oct[o].push_back(e);
        }
        std::vector<int32_t>().swap(list);  // release the parent list early
        nodes.push_back(nd);
        for (int o = 0; o < 8; ++o) {
            if (oct[o].empty()) continue;
            float cmn[3], cmx[3];
            for (int a = 0; a < 3; ++a) {
                const bool upper = (o >> a) & 1;
                cmn[a] = upper ? c[a] : mn[a];
                cmx[a] = upper ? mx[a] : c[a];
            }
            const int32_t ch = subdivide(cmn, cmx, oct[o], depth + 1);
            nodes[idx].children[o] = ch;
        }
        return idx;
    }
};

struct Octree {
    std::vector<Node> nodes;
    std::vector<int32_t> elems;
    std::vector<float> tet_box, tet_geom;
    jt_octree_info info;
};

}  // namespace

extern "C" int jt_octree_build(const float* points, int32_t n_points, const int32_t* conn, int32_t n_tets,
                               int32_t max_elements_per_leaf, int32_t max_depth, void** handle_out,
                               jt_octree_info* info) {
    using jt::set_error;
    if (handle_out == nullptr || info == nullptr) return set_error(JT_ERR_INVALID, "handle_out and info are required");
    *handle_out = nullptr;
    if (points == nullptr || conn == nullptr || n_points < 1 || n_tets < 1)
        return set_error(JT_ERR_INVALID, "octree build needs points and tetrahedra");
    if (max_depth < 0) return set_error(JT_ERR_INVALID, "max_depth must be >= 0");
    for (int64_t k = 0; k < 4LL * n_tets; ++k) {
        if (conn[k] < 0 || conn[k] >= n_points)
            return set_error(JT_ERR_INVALID, "connectivity entry %lld = %d outside [0,%d)", (long long)k, conn[k], n_points);
    }
    Octree* T = new (std::nothrow) Octree();
    if (T == nullptr) return set_error(JT_ERR_NOMEM, "out of host memory");
    try {
        Builder B;
        B.pts = points;
        B.conn = conn;
        B.n_tets = n_tets;
        B.max_per_leaf = max_elements_per_leaf;
        B.max_depth = max_depth;
        B.centroid.resize(3 * (size_t)n_tets);
        T->tet_box.assign(8 * (size_t)n_tets, 0.0f);
        T->tet_geom.assign(16 * (size_t)n_tets, 0.0f);
        for (int32_t e = 0; e < n_tets; ++e) {
            const int32_t* cv = conn + 4 * (size_t)e;
            const float* p[4] = {points + 3 * (size_t)cv[0], points + 3 * (size_t)cv[1], points + 3 * (size_t)cv[2],
                                 points + 3 * (size_t)cv[3]};
            float* bx = &T->tet_box[8 * (size_t)e];
            float* g = &T->tet_geom[16 * (size_t)e];
            for (int a = 0; a < 3; ++a) {
                float lo = p[0][a], hi = p[0][a];
                for (int k = 1; k < 4; ++k) {
                    lo = p[k][a] < lo ? p[k][a] : lo;
                    hi = p[k][a] > hi ? p[k][a] : hi;
                }
                bx[a] = lo;
                bx[4 + a] = hi;
                volatile float s = p[0][a] + p[1][a];
                s = s + p[2][a];
                s = s + p[3][a];
                B.centroid[3 * (size_t)e + a] = s / 4.0f;
                g[a] = p[0][a];
                volatile float d1 = p[1][a] - p[0][a], d2 = p[2][a] - p[0][a], d3 = p[3][a] - p[0][a];
                g[3 + a] = d1;
                g[6 + a] = d2;
                g[9 + a] = d3;
            }
            memcpy(g + 12, cv, 4 * sizeof(int32_t));
        }
        float mn[3], mx[3];
        for (int a = 0; a < 3; ++a) { mn[a] = points[a]; mx[a] = points[a]; }
        for (int32_t i = 1; i < n_points; ++i)
            for (int a = 0; a < 3; ++a) {
                const float v = points[3 * (size_t)i + a];
                mn[a] = v < mn[a] ? v : mn[a];
                mx[a] = v > mx[a] ? v : mx[a];
            }
        std::vector<int32_t> all((size_t)n_tets);
        for (int32_t e = 0; e < n_tets; ++e) all[e] = e;
        B.subdivide(mn, mx, all, 0);
        T->nodes.swap(B.nodes);
        T->elems.swap(B.elems);
        int max_elems = 0, n_leaves = 0;
        for (const Node& nd : T->nodes) {
            if (nd.elem_count > max_elems) max_elems = nd.elem_count;
            n_leaves += nd.leaf ? 1 : 0;
        }
        T->info.n_nodes = (int32_t)T->nodes.size();
        T->info.n_elem_entries = (int32_t)T->elems.size();
        T->info.max_elems = max_elems;
        T->info.max_tree_depth = B.max_leaf_depth;
        T->info.n_leaves = n_leaves;
        T->info.pad = 0;
    } catch (const std::bad_alloc&) {
        delete T;
        return set_error(JT_ERR_NOMEM, "out of host memory during octree build");
    }
    *info = T->info;
    *handle_out = T;
    return JT_OK;
}

extern "C" int jt_octree_fetch(void* handle, jt_octree_node* nodes, int32_t* elems, float* tet_box, float* tet_geom,
                               float* node_bounds) {
    using jt::set_error;
    if (handle == nullptr) return set_error(JT_ERR_INVALID, "octree handle is NULL");
    const Octree* T = static_cast<const Octree*>(handle);
    if (nodes != nullptr) {
        for (size_t i = 0; i < T->nodes.size(); ++i) {
            const Node& s = T->nodes[i];
            jt_octree_node& d = nodes[i];
            float c[3];
            for (int a = 0; a < 3; ++a) {
                volatile float sum = s.mn[a] + s.mx[a];
                c[a] = sum / 2.0f;  // the traversal's centre (…optimized.py:285)
            }
            d.cx = c[0]; d.cy = c[1]; d.cz = c[2];
            d.is_leaf = s.leaf ? 1 : 0;
            for (int o = 0; o < 8; ++o) d.children[o] = s.children[o];
            d.elem_offset = s.elem_offset;
            d.elem_count = s.elem_count;
            d.pad0 = s.depth;
            d.pad1 = 0;
        }
    }
    if (node_bounds != nullptr) {
        for (size_t i = 0; i < T->nodes.size(); ++i)
            for (int a = 0; a < 3; ++a) {
                node_bounds[6 * i + a] = T->nodes[i].mn[a];
                node_bounds[6 * i + 3 + a] = T->nodes[i].mx[a];
            }
    }
    if (elems != nullptr && !T->elems.empty()) memcpy(elems, T->elems.data(), T->elems.size() * sizeof(int32_t));
    if (tet_box != nullptr) memcpy(tet_box, T->tet_box.data(), T->tet_box.size() * sizeof(float));
    if (tet_geom != nullptr) memcpy(tet_geom, T->tet_geom.data(), T->tet_geom.size() * sizeof(float));
    return JT_OK;
}

extern "C" void jt_octree_free(void* handle) { delete static_cast<Octree*>(handle); }
