// Device build of the octree of a tetrahedral mesh, giving the same arrays as
// the host builder (jt_octree.cpp), which follows build_octree_mesh_optimized
// (fields/octree_fem_interpolator_optimized.py:41-215).
//
// The recursion there splits a node's element list by the octant of each
// element's centroid against the node centre, keeps the list order (a stable
// partition of an ascending list), and numbers nodes in DFS pre-order with
// octants 0..7.  Here the tree grows one level per pass with the elements
// left in place:
//   * each element carries its current node; a pass gives it an octant digit
//     and counts the digits per node (warp-aggregated atomics);
//   * a scan over the level's nodes numbers the non-empty octants as the
//     next level's nodes (breadth-first ids), with box, count and leaf flag
//     (count <= max_elements_per_leaf or depth >= max_depth);
//   * elements of nodes that became leaves stop; the rest step down.
// Afterwards subtree sizes (bottom-up) give every node its DFS pre-order id
// and its element offset (top-down: the parent's, plus the counts of the
// earlier octants), elements are scattered into their leaves' ranges and each
// leaf's range is sorted ascending -- exactly the order the stable recursive
// partition leaves, since it starts from the ascending list 0..n-1.
// Float32 arithmetic matches the host: centroid ((p0+p1)+p2)+p3 then /4,
// node centre (min+max)/2, each operation rounded.
#include <stdint.h>

#include <new>
#include <vector>

#include "jt_internal.h"
#include "jt_mesh.cuh"

namespace jt {

constexpr int kOctBlock = 256;

__global__ void __launch_bounds__(kOctBlock) k_mark_near_degenerate(float* __restrict__ tet_box,
                                                                    const float* __restrict__ tet_geom, int n_tets,
                                                                    int* __restrict__ count) {
    const int t = blockIdx.x * kOctBlock + threadIdx.x;
    if (t >= n_tets) return;
    const bool near = near_degenerate(tet_geom + 16 * (int64_t)t);
    tet_box[8 * (int64_t)t + 3] = near ? 1.0f : 0.0f;
    if (near) atomicAdd(count, 1);
}

__device__ __forceinline__ float oct_centre(float mn, float mx) { return __fmul_rn(__fadd_rn(mn, mx), 0.5f); }

// per-block min/max of the points (host order: v < mn ? v : mn)
__global__ void __launch_bounds__(kOctBlock) k_oct_bounds(const float* __restrict__ pts, int n,
                                                          float* __restrict__ part) {
    __shared__ float s[6][kOctBlock];
    float mn[3], mx[3];
    for (int a = 0; a < 3; ++a) {
        mn[a] = pts[a];
        mx[a] = pts[a];
    }
    for (int i = blockIdx.x * kOctBlock + threadIdx.x; i < n; i += gridDim.x * kOctBlock)
        for (int a = 0; a < 3; ++a) {
            const float v = pts[3 * (int64_t)i + a];
            mn[a] = v < mn[a] ? v : mn[a];
            mx[a] = v > mx[a] ? v : mx[a];
        }
    for (int a = 0; a < 3; ++a) {
        s[a][threadIdx.x] = mn[a];
        s[3 + a][threadIdx.x] = mx[a];
    }
    __syncthreads();
    for (int w = kOctBlock / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int a = 0; a < 3; ++a) {
                const float l = s[a][threadIdx.x + w], h = s[3 + a][threadIdx.x + w];
                s[a][threadIdx.x] = l < s[a][threadIdx.x] ? l : s[a][threadIdx.x];
                s[3 + a][threadIdx.x] = h > s[3 + a][threadIdx.x] ? h : s[3 + a][threadIdx.x];
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void k_oct_bounds_final(const float* __restrict__ part, int nb, float* __restrict__ box) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float b[6];
    for (int a = 0; a < 6; ++a) b[a] = part[a];
    for (int k = 1; k < nb; ++k)
        for (int a = 0; a < 3; ++a) {
            const float l = part[6 * k + a], h = part[6 * k + 3 + a];
            b[a] = l < b[a] ? l : b[a];
            b[3 + a] = h > b[3 + a] ? h : b[3 + a];
        }
    for (int a = 0; a < 6; ++a) box[a] = b[a];
}

// per-tetrahedron box (min xyz,0,max xyz,0), geometry (v0, v1-v0, v2-v0,
// v3-v0, vertex ids) and centroid; connectivity outside the points sets *bad
__global__ void __launch_bounds__(kOctBlock) k_oct_tets(const float* __restrict__ pts, const int32_t* __restrict__ conn,
                                                        int n_tets, int n_points, float* __restrict__ tet_box,
                                                        float* __restrict__ tet_geom, float* __restrict__ cen,
                                                        int* __restrict__ bad) {
    const int e = blockIdx.x * kOctBlock + threadIdx.x;
    if (e >= n_tets) return;
    int v[4];
    for (int k = 0; k < 4; ++k) {
        v[k] = conn[4 * (int64_t)e + k];
        if (v[k] < 0 || v[k] >= n_points) {
            atomicExch(bad, 1);
            v[k] = 0;
        }
    }
    for (int a = 0; a < 3; ++a) {
        float p[4];
        for (int k = 0; k < 4; ++k) p[k] = pts[3 * (int64_t)v[k] + a];
        float lo = p[0], hi = p[0];
        for (int k = 1; k < 4; ++k) {
            lo = p[k] < lo ? p[k] : lo;
            hi = p[k] > hi ? p[k] : hi;
        }
        cen[3 * (int64_t)e + a] = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(p[0], p[1]), p[2]), p[3]), 0.25f);
        if (tet_box != nullptr) {
            tet_box[8 * (int64_t)e + a] = lo;
            tet_box[8 * (int64_t)e + 4 + a] = hi;
        }
        if (tet_geom != nullptr) {
            float* g = tet_geom + 16 * (int64_t)e;
            g[a] = p[0];
            g[3 + a] = __fsub_rn(p[1], p[0]);
            g[6 + a] = __fsub_rn(p[2], p[0]);
            g[9 + a] = __fsub_rn(p[3], p[0]);
        }
    }
    if (tet_box != nullptr) {
        tet_box[8 * (int64_t)e + 3] = 0.0f;
        tet_box[8 * (int64_t)e + 7] = 0.0f;
    }
    if (tet_geom != nullptr)
        for (int k = 0; k < 4; ++k) tet_geom[16 * (int64_t)e + 12 + k] = __int_as_float(conn[4 * (int64_t)e + k]);
}

__global__ void __launch_bounds__(kOctBlock) k_oct_init(int n, int root_internal, int* __restrict__ cur,
                                                        int* __restrict__ leaf_of) {
    const int e = blockIdx.x * kOctBlock + threadIdx.x;
    if (e >= n) return;
    cur[e] = root_internal ? 0 : -1;
    leaf_of[e] = 0;
}

// octant digit of every element still descending, counted per (node, octant)
__global__ void __launch_bounds__(kOctBlock) k_oct_digits(int n, const float* __restrict__ cen,
                                                          const int* __restrict__ cur, const float* __restrict__ box,
                                                          unsigned char* __restrict__ digit, int* __restrict__ ccount) {
    const int e = blockIdx.x * kOctBlock + threadIdx.x;
    const int j = e < n ? cur[e] : -1;
    int key = -1;
    if (j >= 0) {
        const float* b = box + 6 * (int64_t)j;
        int o = 0;
        if (cen[3 * (int64_t)e] >= oct_centre(b[0], b[3])) o += 1;
        if (cen[3 * (int64_t)e + 1] >= oct_centre(b[1], b[4])) o += 2;
        if (cen[3 * (int64_t)e + 2] >= oct_centre(b[2], b[5])) o += 4;
        digit[e] = (unsigned char)o;
        key = 8 * j + o;
    }
    // one atomic per distinct key in the warp
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&ccount[key], __popc(peers));
}

__global__ void __launch_bounds__(kOctBlock) k_oct_nchild(int m, const int* __restrict__ ccount,
                                                          int* __restrict__ nchild) {
    const int j = blockIdx.x * kOctBlock + threadIdx.x;
    if (j >= m) return;
    int c = 0;
    for (int o = 0; o < 8; ++o) c += ccount[8 * j + o] > 0;
    nchild[j] = c;
}

// in-place exclusive scan of a[0..m) by one block; *total = the sum
__global__ void __launch_bounds__(1024) k_oct_scan(int* __restrict__ a, int m, int* __restrict__ total) {
    __shared__ int s[1024];
    int carry = 0;
    for (int base = 0; base < m; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < m ? a[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int w = 1; w < 1024; w <<= 1) {
            const int t = threadIdx.x >= w ? s[threadIdx.x - w] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < m) a[i] = carry + s[threadIdx.x] - v;
        const int tile = s[1023];
        __syncthreads();
        carry += tile;
    }
    if (threadIdx.x == 0) *total = carry;
}

// the next level's nodes; stats = {internal children, leaves, longest leaf}
__global__ void __launch_bounds__(kOctBlock) k_oct_children(int m, const float* __restrict__ box,
                                                            const int* __restrict__ ccount,
                                                            const int* __restrict__ base, int depth_next, int mpl,
                                                            int max_depth, int* __restrict__ child,
                                                            float* __restrict__ nbox, int* __restrict__ ncount,
                                                            int* __restrict__ nleaf, int* __restrict__ stats) {
    const int j = blockIdx.x * kOctBlock + threadIdx.x;
    if (j >= m) return;
    const float* b = box + 6 * (int64_t)j;
    float c[3];
    for (int a = 0; a < 3; ++a) c[a] = oct_centre(b[a], b[3 + a]);
    int k = base[j];
    for (int o = 0; o < 8; ++o) {
        const int cnt = ccount[8 * j + o];
        if (cnt == 0) {
            child[8 * j + o] = -1;
            continue;
        }
        float* nb = nbox + 6 * (int64_t)k;
        for (int a = 0; a < 3; ++a) {
            const bool upper = (o >> a) & 1;
            nb[a] = upper ? c[a] : b[a];
            nb[3 + a] = upper ? b[3 + a] : c[a];
        }
        const bool leaf = cnt <= mpl || depth_next >= max_depth;
        ncount[k] = cnt;
        nleaf[k] = leaf ? 1 : 0;
        if (leaf) {
            atomicAdd(&stats[1], 1);
            atomicMax(&stats[2], cnt);
        } else {
            atomicAdd(&stats[0], 1);
        }
        child[8 * j + o] = k;
        ++k;
    }
}

__global__ void __launch_bounds__(kOctBlock) k_oct_advance(int n, int* __restrict__ cur,
                                                           const unsigned char* __restrict__ digit,
                                                           const int* __restrict__ child, const int* __restrict__ nleaf,
                                                           int next_base, int* __restrict__ leaf_of) {
    const int e = blockIdx.x * kOctBlock + threadIdx.x;
    if (e >= n) return;
    const int j = cur[e];
    if (j < 0) return;
    const int k = child[8 * j + digit[e]];
    if (nleaf[k]) {
        leaf_of[e] = next_base + k;
        cur[e] = -1;
    } else {
        cur[e] = k;
    }
}

// subtree node counts, deepest level first
__global__ void __launch_bounds__(kOctBlock) k_oct_size(int m, const int* __restrict__ child,
                                                        const int* __restrict__ size_next, int* __restrict__ size) {
    const int j = blockIdx.x * kOctBlock + threadIdx.x;
    if (j >= m) return;
    int s = 1;
    if (size_next != nullptr)
        for (int o = 0; o < 8; ++o) {
            const int k = child[8 * j + o];
            if (k >= 0) s += size_next[k];
        }
    size[j] = s;
}

// DFS pre-order ids and element offsets of the next level, from this level's
__global__ void __launch_bounds__(kOctBlock) k_oct_dfs(int m, const int* __restrict__ child,
                                                       const int* __restrict__ dfs, const int* __restrict__ off,
                                                       const int* __restrict__ size_next,
                                                       const int* __restrict__ count_next, int* __restrict__ dfs_next,
                                                       int* __restrict__ off_next) {
    const int j = blockIdx.x * kOctBlock + threadIdx.x;
    if (j >= m) return;
    int r = dfs[j] + 1, eo = off[j];
    for (int o = 0; o < 8; ++o) {
        const int k = child[8 * j + o];
        if (k < 0) continue;
        dfs_next[k] = r;
        off_next[k] = eo;
        r += size_next[k];
        eo += count_next[k];
    }
}

__global__ void __launch_bounds__(kOctBlock) k_oct_write(int m, int depth, int flat_base, const float* __restrict__ box,
                                                         const int* __restrict__ count, const int* __restrict__ leaf,
                                                         const int* __restrict__ child, const int* __restrict__ dfs,
                                                         const int* __restrict__ off, const int* __restrict__ dfs_next,
                                                         jt_octree_node* __restrict__ nodes, float* __restrict__ bounds,
                                                         int* __restrict__ flat_off, int* __restrict__ flat_cnt) {
    const int j = blockIdx.x * kOctBlock + threadIdx.x;
    if (j >= m) return;
    const int d = dfs[j];
    const float* b = box + 6 * (int64_t)j;
    jt_octree_node nd;
    nd.cx = oct_centre(b[0], b[3]);
    nd.cy = oct_centre(b[1], b[4]);
    nd.cz = oct_centre(b[2], b[5]);
    nd.is_leaf = leaf[j];
    for (int o = 0; o < 8; ++o) {
        const int k = child[8 * j + o];
        nd.children[o] = k >= 0 ? dfs_next[k] : -1;
    }
    nd.elem_offset = off[j];
    nd.elem_count = leaf[j] ? count[j] : 0;
    nd.pad0 = depth;
    nd.pad1 = 0;
    nodes[d] = nd;
    if (bounds != nullptr)
        for (int a = 0; a < 6; ++a) bounds[6 * (int64_t)d + a] = b[a];
    flat_off[flat_base + j] = off[j];
    flat_cnt[flat_base + j] = nd.elem_count;
}

__global__ void __launch_bounds__(kOctBlock) k_oct_scatter(int n, const int* __restrict__ leaf_of,
                                                           const int* __restrict__ flat_off, int* __restrict__ cursor,
                                                           int* __restrict__ tmp) {
    const int e = blockIdx.x * kOctBlock + threadIdx.x;
    if (e >= n) return;
    const int l = leaf_of[e];
    tmp[flat_off[l] + atomicAdd(&cursor[l], 1)] = e;
}

// one warp per node: its leaf range sorted ascending by rank (ids are distinct)
__global__ void __launch_bounds__(kOctBlock) k_oct_sort_leaves(int n_flat, const int* __restrict__ flat_off,
                                                               const int* __restrict__ flat_cnt,
                                                               const int* __restrict__ tmp, int* __restrict__ elems) {
    const int w = (blockIdx.x * kOctBlock + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n_flat) return;
    const int c = flat_cnt[w];
    if (c == 0) return;
    const int* src = tmp + flat_off[w];
    for (int i = lane; i < c; i += 32) {
        const int v = src[i];
        int rank = 0;
        for (int q = 0; q < c; ++q) rank += src[q] < v;
        elems[flat_off[w] + rank] = v;
    }
}

}  // namespace jt

using namespace jt;

namespace {

struct DevOctree {
    jt_octree_node* nodes = nullptr;
    float* bounds = nullptr;
    int32_t n_nodes = 0;
};

struct Level {
    int m = 0;
    float* box = nullptr;   // (m,6)
    int* count = nullptr;   // (m)
    int* leaf = nullptr;    // (m)
    int* ccount = nullptr;  // (m,8) digit counts
    int* child = nullptr;   // (m,8) next-level ids, -1 empty
    int* size = nullptr;
    int* dfs = nullptr;
    int* off = nullptr;
};

// device allocations of one build, released together on the stream
struct Pool {
    cudaStream_t s;
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <class T>
    T* get(size_t n) {
        void* p = nullptr;
        if (err == cudaSuccess) err = dev_alloc(&p, n * sizeof(T) > 0 ? n * sizeof(T) : 16, s);
        if (err != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    ~Pool() {
        for (void* p : ptrs) dev_free(p, s);
    }
};

inline unsigned blocks(int64_t n) { return (unsigned)((n + kOctBlock - 1) / kOctBlock); }

}  // namespace

extern "C" int jt_octree_build_device(const float* points, int32_t n_points, const int32_t* conn, int32_t n_tets,
                                      int32_t max_elements_per_leaf, int32_t max_depth, int32_t* elems,
                                      float* tet_box, float* tet_geom, void* stream, void** handle_out,
                                      jt_octree_info* info) {
    if (handle_out == nullptr || info == nullptr) return set_error(JT_ERR_INVALID, "handle_out and info are required");
    *handle_out = nullptr;
    if (points == nullptr || conn == nullptr || elems == nullptr || n_points < 1 || n_tets < 1)
        return set_error(JT_ERR_INVALID, "octree build needs points, tetrahedra and an elems buffer");
    if (max_depth < 0) return set_error(JT_ERR_INVALID, "max_depth must be >= 0");
    if (max_depth > 40) return set_error(JT_ERR_INVALID, "max_depth must be <= 40");
    cudaStream_t s = (cudaStream_t)stream;
    Pool pool{s};
    const int n = n_tets;
    const unsigned nbb = 152;
    float* part = pool.get<float>(6 * nbb);
    float* root_box = pool.get<float>(6);
    float* cen = pool.get<float>(3 * (size_t)n);
    int* cur = pool.get<int>(n);
    int* leaf_of = pool.get<int>(n);
    unsigned char* digit = pool.get<unsigned char>(n);
    int* scal = pool.get<int>(8);  // [0] bad connectivity, [1] scan total, [2..4] stats
    if (pool.err != cudaSuccess) return cuda_status(pool.err, "octree build allocation");
    cudaError_t e = cudaMemsetAsync(scal, 0, 8 * sizeof(int), s);
    if (e != cudaSuccess) return cuda_status(e, "octree build reset");
    k_oct_bounds<<<nbb, kOctBlock, 0, s>>>(points, n_points, part);
    k_oct_bounds_final<<<1, 32, 0, s>>>(part, (int)nbb, root_box);
    k_oct_tets<<<blocks(n), kOctBlock, 0, s>>>(points, conn, n, n_points, tet_box, tet_geom, cen, scal);
    const bool root_internal = !(n <= max_elements_per_leaf || max_depth <= 0);
    k_oct_init<<<blocks(n), kOctBlock, 0, s>>>(n, root_internal ? 1 : 0, cur, leaf_of);
    std::vector<Level> lv(1);
    lv[0].m = 1;
    lv[0].box = root_box;
    lv[0].count = pool.get<int>(1);
    lv[0].leaf = pool.get<int>(1);
    if (pool.err != cudaSuccess) return cuda_status(pool.err, "octree build allocation");
    {
        const int h[2] = {n, root_internal ? 0 : 1};
        if ((e = cudaMemcpyAsync(lv[0].count, &h[0], sizeof(int), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(lv[0].leaf, &h[1], sizeof(int), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return cuda_status(e, "octree build root");
    }
    int host_bad = 0;
    if ((e = cudaMemcpy(&host_bad, scal, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_status(e, "octree build check");
    if (host_bad) return set_error(JT_ERR_INVALID, "connectivity indexes outside the points array");
    int n_leaves = root_internal ? 0 : 1, max_elems = root_internal ? 0 : n;
    int internal = root_internal ? 1 : 0;
    // one level per pass while internal nodes remain
    for (int depth = 0; internal > 0; ++depth) {
        Level& L = lv[depth];
        L.ccount = pool.get<int>(8 * (size_t)L.m);
        L.child = pool.get<int>(8 * (size_t)L.m);
        int* nchild = pool.get<int>(L.m);
        if (pool.err != cudaSuccess) return cuda_status(pool.err, "octree level allocation");
        if ((e = cudaMemsetAsync(L.ccount, 0, 8 * sizeof(int) * (size_t)L.m, s)) != cudaSuccess ||
            (e = cudaMemsetAsync(scal + 2, 0, 3 * sizeof(int), s)) != cudaSuccess)
            return cuda_status(e, "octree level reset");
        k_oct_digits<<<blocks(n), kOctBlock, 0, s>>>(n, cen, cur, L.box, digit, L.ccount);
        k_oct_nchild<<<blocks(L.m), kOctBlock, 0, s>>>(L.m, L.ccount, nchild);
        k_oct_scan<<<1, 1024, 0, s>>>(nchild, L.m, scal + 1);
        int m_next = 0;
        if ((e = cudaMemcpyAsync(&m_next, scal + 1, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return cuda_status(e, "octree level count");
        Level N;
        N.m = m_next;
        N.box = pool.get<float>(6 * (size_t)m_next);
        N.count = pool.get<int>(m_next);
        N.leaf = pool.get<int>(m_next);
        if (pool.err != cudaSuccess) return cuda_status(pool.err, "octree level allocation");
        k_oct_children<<<blocks(L.m), kOctBlock, 0, s>>>(L.m, L.box, L.ccount, nchild, depth + 1,
                                                         max_elements_per_leaf, max_depth, L.child, N.box, N.count,
                                                         N.leaf, scal + 2);
        int next_base = 0;
        for (const Level& q : lv) next_base += q.m;
        k_oct_advance<<<blocks(n), kOctBlock, 0, s>>>(n, cur, digit, L.child, N.leaf, next_base, leaf_of);
        int st[3];
        if ((e = cudaMemcpyAsync(st, scal + 2, 3 * sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return cuda_status(e, "octree level stats");
        internal = st[0];
        n_leaves += st[1];
        max_elems = st[2] > max_elems ? st[2] : max_elems;
        lv.push_back(N);
    }
    const int n_levels = (int)lv.size();
    int64_t total = 0;
    for (const Level& q : lv) total += q.m;
    if (total > INT32_MAX) return set_error(JT_ERR_NOMEM, "octree node count exceeds 2^31");
    const int n_nodes = (int)total;
    // subtree sizes bottom-up, then DFS ids and offsets top-down
    for (int d = n_levels - 1; d >= 0; --d) {
        Level& L = lv[d];
        L.size = pool.get<int>(L.m);
        L.dfs = pool.get<int>(L.m);
        L.off = pool.get<int>(L.m);
        if (pool.err != cudaSuccess) return cuda_status(pool.err, "octree order allocation");
        if (L.child == nullptr) {  // deepest level: all leaves, no children
            L.child = pool.get<int>(8 * (size_t)L.m);
            if (pool.err != cudaSuccess) return cuda_status(pool.err, "octree order allocation");
            if ((e = cudaMemsetAsync(L.child, 0xff, 8 * sizeof(int) * (size_t)L.m, s)) != cudaSuccess)
                return cuda_status(e, "octree order reset");
        }
        k_oct_size<<<blocks(L.m), kOctBlock, 0, s>>>(L.m, L.child, d + 1 < n_levels ? lv[d + 1].size : nullptr,
                                                     L.size);
    }
    if ((e = cudaMemsetAsync(lv[0].dfs, 0, sizeof(int), s)) != cudaSuccess ||
        (e = cudaMemsetAsync(lv[0].off, 0, sizeof(int), s)) != cudaSuccess)
        return cuda_status(e, "octree order root");
    for (int d = 0; d + 1 < n_levels; ++d)
        k_oct_dfs<<<blocks(lv[d].m), kOctBlock, 0, s>>>(lv[d].m, lv[d].child, lv[d].dfs, lv[d].off, lv[d + 1].size,
                                                         lv[d + 1].count, lv[d + 1].dfs, lv[d + 1].off);
    DevOctree* T = new (std::nothrow) DevOctree();
    if (T == nullptr) return set_error(JT_ERR_NOMEM, "out of host memory");
    T->n_nodes = n_nodes;
    if ((e = dev_alloc((void**)&T->nodes, sizeof(jt_octree_node) * (size_t)n_nodes, s)) != cudaSuccess ||
        (e = dev_alloc((void**)&T->bounds, 6 * sizeof(float) * (size_t)n_nodes, s)) != cudaSuccess) {
        if (T->nodes) dev_free(T->nodes, s);
        delete T;
        return cuda_status(e, "octree node allocation");
    }
    int* flat_off = pool.get<int>(n_nodes);
    int* flat_cnt = pool.get<int>(n_nodes);
    int* cursor = pool.get<int>(n_nodes);
    int* tmp = pool.get<int>(n);
    if (pool.err == cudaSuccess) e = cudaMemsetAsync(cursor, 0, sizeof(int) * (size_t)n_nodes, s);
    if (pool.err != cudaSuccess || e != cudaSuccess) {
        dev_free(T->nodes, s);
        dev_free(T->bounds, s);
        delete T;
        return cuda_status(pool.err != cudaSuccess ? pool.err : e, "octree element allocation");
    }
    int flat_base = 0;
    for (int d = 0; d < n_levels; ++d) {
        const Level& L = lv[d];
        k_oct_write<<<blocks(L.m), kOctBlock, 0, s>>>(L.m, d, flat_base, L.box, L.count, L.leaf, L.child, L.dfs,
                                                      L.off, d + 1 < n_levels ? lv[d + 1].dfs : L.dfs, T->nodes,
                                                      T->bounds, flat_off, flat_cnt);
        flat_base += L.m;
    }
    k_oct_scatter<<<blocks(n), kOctBlock, 0, s>>>(n, leaf_of, flat_off, cursor, tmp);
    k_oct_sort_leaves<<<blocks((int64_t)n_nodes * 32), kOctBlock, 0, s>>>(n_nodes, flat_off, flat_cnt, tmp, elems);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        dev_free(T->nodes, s);
        dev_free(T->bounds, s);
        delete T;
        return cuda_status(e, "octree build kernels");
    }
    info->n_nodes = n_nodes;
    info->n_elem_entries = n;
    info->max_elems = max_elems;
    info->max_tree_depth = n_levels - 1;
    info->n_leaves = n_leaves;
    info->pad = 0;
    *handle_out = T;
    return JT_OK;
}

extern "C" int jt_octree_fetch_device(void* handle, jt_octree_node* nodes, float* node_bounds, void* stream) {
    if (handle == nullptr) return set_error(JT_ERR_INVALID, "octree handle is NULL");
    const DevOctree* T = static_cast<const DevOctree*>(handle);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (nodes != nullptr)
        e = cudaMemcpyAsync(nodes, T->nodes, sizeof(jt_octree_node) * (size_t)T->n_nodes, cudaMemcpyDefault, s);
    if (e == cudaSuccess && node_bounds != nullptr)
        e = cudaMemcpyAsync(node_bounds, T->bounds, 6 * sizeof(float) * (size_t)T->n_nodes, cudaMemcpyDefault, s);
    return cuda_status(e, "octree fetch");
}

extern "C" void jt_octree_free_device(void* handle, void* stream) {
    DevOctree* T = static_cast<DevOctree*>(handle);
    if (T == nullptr) return;
    cudaStream_t s = (cudaStream_t)stream;
    dev_free(T->nodes, s);
    dev_free(T->bounds, s);
    delete T;
}

extern "C" int jt_mark_near_degenerate(float* tet_box, const float* tet_geom, int32_t n_tets, int32_t* count_out,
                                       void* stream) {
    if (n_tets < 0) return set_error(JT_ERR_INVALID, "n_tets must be >= 0");
    if (n_tets > 0 && (tet_box == nullptr || tet_geom == nullptr))
        return set_error(JT_ERR_INVALID, "tet_box and tet_geom are required");
    cudaStream_t s = (cudaStream_t)stream;
    int* d = nullptr;
    cudaError_t e = dev_alloc((void**)&d, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(int), s);
    if (e == cudaSuccess && n_tets > 0) {
        k_mark_near_degenerate<<<(unsigned)((n_tets + kOctBlock - 1) / kOctBlock), kOctBlock, 0, s>>>(tet_box, tet_geom,
                                                                                                   n_tets, d);
        e = cudaGetLastError();
    }
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (d != nullptr) dev_free(d, s);
    if (e != cudaSuccess) return cuda_status(e, "near-degenerate marking");
    if (count_out != nullptr) *count_out = h;
    return JT_OK;
}
