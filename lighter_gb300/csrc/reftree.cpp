// Host build of the reference-shaped per-instance trees (see reftree.hpp).
#include "reftree.hpp"

#include "../../include/lighter_gb300.h"

#include <algorithm>
#include <cfloat>
#include <exception>
#include <thread>

namespace lg {
namespace {

struct Box { V3 mn, mx; };

inline float volume(const Box& b) { return (b.mx.x - b.mn.x) * (b.mx.y - b.mn.y) * (b.mx.z - b.mn.z); }
inline V3 centre(const Box& b) { return (b.mn + b.mx) * 0.5f; }

// Subtrees of at least kParItems items above depth kParDepth are built on a
// second thread into a separate tree and spliced in afterwards (node and item
// offsets shifted), which gives the sequential build's layout exactly.
constexpr size_t kParItems = 1024;
constexpr int kParDepth = 4;

struct Builder {
    const Box* boxes;
    RefTree* t;
    int par_depth;   // levels whose halves are built on two threads (kParDepth, or -1: none)

    // Appends `sub` (built with its root at index 0 and its own item list) as the
    // subtree whose root gets the next node index.
    void splice(const RefTree& sub)
    {
        const int32_t nb = (int32_t) t->nodes.size(), ib = (int32_t) t->items.size();
        for (RefNode nd : sub.nodes) {
            if (nd.ch != -1) nd.ch += nb;
            if (nd.ido != -1) nd.ido += ib;
            t->nodes.push_back(nd);
        }
        t->items.insert(t->items.end(), sub.items.begin(), sub.items.end());
    }

    void emit(int32_t node, const int32_t* ids, size_t n)
    {
        t->nodes[node].ido = (int32_t) t->items.size();
        t->items.push_back((int32_t) n);
        t->items.insert(t->items.end(), ids, ids + n);
    }

    void make(int32_t node, const int32_t* ids, size_t n, int depth)
    {
        V3 mn = splat(FLT_MAX), mx = splat(-FLT_MAX);
        for (size_t i = 0; i < n; ++i) { mn = vmin(mn, boxes[ids[i]].mn); mx = vmax(mx, boxes[ids[i]].mx); }
        RefNode& N = t->nodes[node];
        N.mn[0] = mn.x; N.mn[1] = mn.y; N.mn[2] = mn.z;
        N.mx[0] = mx.x; N.mx[1] = mx.y; N.mx[2] = mx.z;
        N.ch = -1;
        N.ido = -1;
        Box nb = {mn, mx};
        float nvol = volume(nb);
        if (n > 4 && depth < 16) {
            int nsplit = 0;
            V3 smn = splat(FLT_MAX), smx = splat(-FLT_MAX);
            for (size_t i = 0; i < n; ++i) {
                const Box& b = boxes[ids[i]];
                if (volume(b) * 3 < nvol) { nsplit++; smn = vmin(smn, b.mn); smx = vmax(smx, b.mx); }
            }
            V3 ss = smx - smn;
            V3 axis = mk(0, 0, 1);
            if (ss.x > ss.y && ss.x > ss.z) axis = mk(1, 0, 0);
            else if (ss.y > ss.x && ss.y > ss.z) axis = mk(0, 1, 0);
            if (nsplit >= 4) {
                std::vector<int32_t> self, split;
                for (size_t i = 0; i < n; ++i) {
                    if (volume(boxes[ids[i]]) * 3 < nvol) split.push_back(ids[i]);
                    else self.push_back(ids[i]);
                }
                if (!self.empty()) emit(node, self.data(), self.size());
                // the keys are the values the comparison dot(axis, centre(a)) < dot(axis,
                // centre(b)) would compute, so std::sort sees the same comparisons;
                // sorting (key, id) pairs makes the same comparisons in the same
                // sequence, so it gives the same order, without the indirection
                std::vector<std::pair<float, int32_t>> kp(split.size());
                for (size_t i = 0; i < split.size(); ++i) kp[i] = {dot(axis, centre(boxes[split[i]])), split[i]};
                std::sort(kp.begin(), kp.end(), [](const std::pair<float, int32_t>& a, const std::pair<float, int32_t>& b) {
                    return a.first < b.first;
                });
                for (size_t i = 0; i < split.size(); ++i) split[i] = kp[i].second;
                size_t mid = split.size() / 2;
                if (depth < par_depth && split.size() >= kParItems) {
                    // both halves at once: the right one on a second thread
                    RefTree right;
                    right.nodes.assign(1, RefNode());
                    Builder rb{boxes, &right, par_depth};
                    std::exception_ptr rerr;
                    std::thread th([&]() {
                        try {
                            rb.make(0, split.data() + mid, split.size() - mid, depth + 1);
                        } catch (...) {
                            rerr = std::current_exception();
                        }
                    });
                    RefTree left;
                    left.nodes.assign(1, RefNode());
                    Builder lb{boxes, &left, par_depth};
                    try {
                        lb.make(0, split.data(), mid, depth + 1);
                    } catch (...) {
                        th.join();
                        throw;
                    }
                    th.join();
                    if (rerr) std::rethrow_exception(rerr);
                    splice(left);
                    t->nodes[node].ch = (int32_t) t->nodes.size();
                    splice(right);
                    return;
                }
                t->nodes.push_back(RefNode());
                make((int32_t) t->nodes.size() - 1, split.data(), mid, depth + 1);
                t->nodes[node].ch = (int32_t) t->nodes.size();
                t->nodes.push_back(RefNode());
                make((int32_t) t->nodes.size() - 1, split.data() + mid, split.size() - mid, depth + 1);
                return;
            }
        }
        emit(node, ids, n);
    }
};

}  // namespace

void build_ref_tree(const float* xyz, size_t n, RefTree& out, bool threads)
{
    out.nodes.assign(1, RefNode());
    out.items.clear();
    RefNode& root = out.nodes[0];
    for (int c = 0; c < 3; ++c) { root.mn[c] = FLT_MAX; root.mx[c] = -FLT_MAX; }
    root.ch = -1;
    root.ido = -1;
    if (n == 0) return;
    std::vector<Box> boxes(n);
    std::vector<int32_t> ids;
    ids.reserve(n);
    for (size_t i = 0; i < n; ++i) {
        const float* p = xyz + 9 * i;
        V3 a = mk(p[0], p[1], p[2]), b = mk(p[3], p[4], p[5]), c = mk(p[6], p[7], p[8]);
        boxes[i].mn = vmin(a, vmin(b, c));
        boxes[i].mx = vmax(a, vmax(b, c));
        const Box& bb = boxes[i];
        if (bb.mn.x <= bb.mx.x && bb.mn.y <= bb.mx.y && bb.mn.z <= bb.mx.z) ids.push_back((int32_t) i);
    }
    Builder bld{boxes.data(), &out, threads ? kParDepth : -1};
    bld.make(0, ids.data(), ids.size(), 0);
}

}  // namespace lg

extern "C" LTRAPI LTRBOOL ltrdbg_RefTreeDigest(const float* tri_xyz, u32 n_tris, int threads, uint64_t* out3)
{
    if ((!tri_xyz && n_tris) || !out3) return 0;
    try {
        lg::RefTree t;
        lg::build_ref_tree(tri_xyz, n_tris, t, threads != 0);
        uint64_t h = 1469598103934665603ull;   // FNV-1a over the node and item arrays
        auto mix = [&](const void* p, size_t bytes) {
            const unsigned char* c = (const unsigned char*) p;
            for (size_t i = 0; i < bytes; ++i) { h ^= c[i]; h *= 1099511628211ull; }
        };
        mix(t.nodes.data(), t.nodes.size() * sizeof(lg::RefNode));
        mix(t.items.data(), t.items.size() * sizeof(int32_t));
        out3[0] = t.nodes.size();
        out3[1] = t.items.size();
        out3[2] = h;
    } catch (...) {
        return 0;
    }
    return 1;
}
