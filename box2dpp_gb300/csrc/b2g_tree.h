// Host copy of the reference broadphase's dynamic AABB tree (Box2D 2.3.2 Collision/b2DynamicTree.cpp),
// kept only for b2World::GetTreeHeight, GetTreeBalance and GetTreeQuality (Dynamics/b2World.cpp:
// 1246-1259). The device step never reads a tree: its pair finding works on the fat boxes, and proxy
// ids follow from the tree's free list alone. The tree's shape, however, is the history of every leaf
// insertion and removal, so a world that answers these three calls replays that history here: the
// proxies created and destroyed on the host, and every re-insertion the device makes (MoveProxy when a
// swept box leaves its fat box), which the step logs in the reference's order.
#pragma once

#include <cstring>
#include <vector>

#include "b2g_core.h"

namespace b2g {

class ProxyTree {
public:
    static constexpr int kNone = -1;

    // b2DynamicTree::CreateProxy (:97-131) with the fat box already computed: a pool node for the
    // leaf, then InsertLeaf. Returns the node id, which is the proxy id.
    int Insert(float4 fat)
    {
        const int id = Allocate();
        nodes_[id].box = fat;
        nodes_[id].height = 0;
        InsertLeaf(id);
        return id;
    }
    // b2DynamicTree::DestroyProxy (:124-130)
    void Remove(int id)
    {
        RemoveLeaf(id);
        Release(id);
    }
    // b2DynamicTree::MoveProxy (:133-177) after its containment test failed: out and back in with the
    // new fat box.
    void Move(int id, float4 fat)
    {
        RemoveLeaf(id);
        nodes_[id].box = fat;
        InsertLeaf(id);
    }
    // b2DynamicTree::GetHeight (:523-531)
    int Height() const { return root_ == kNone ? 0 : nodes_[root_].height; }
    // b2DynamicTree::GetMaxBalance (:675-697): over the whole pool, internal nodes above height 1
    int MaxBalance() const
    {
        int best = 0;
        for (const Node& n : nodes_) {
            if (n.height <= 1) continue;
            const int d = nodes_[n.child2].height - nodes_[n.child1].height;
            const int a = d < 0 ? -d : d;
            if (a > best) best = a;
        }
        return best;
    }
    // b2DynamicTree::GetAreaRatio (:534-559): every allocated node's perimeter, summed in pool
    // order, over the root's perimeter
    float AreaRatio() const
    {
        if (root_ == kNone) return 0.0f;
        const float rootP = Perimeter(nodes_[root_].box);
        float sum = 0.0f;
        for (const Node& n : nodes_)
            if (n.height >= 0) sum += Perimeter(n.box);
        return sum / rootP;
    }

    // b2DynamicTree::ShiftOrigin (:773-781): every node box of the pool moves by -origin
    void ShiftOrigin(float x, float y)
    {
        for (Node& n : nodes_) {
            n.box.x = n.box.x - x;
            n.box.y = n.box.y - y;
            n.box.z = n.box.z - x;
            n.box.w = n.box.w - y;
        }
    }

    // the whole tree as bytes (world checkpoints) and back; Load returns false on malformed input
    void Save(std::vector<unsigned char>& out) const
    {
        const int head[3] = {(int)nodes_.size(), root_, free_};
        Append(out, head, sizeof(head));
        if (!nodes_.empty()) Append(out, nodes_.data(), nodes_.size() * sizeof(Node));
    }
    bool Load(const unsigned char*& p, const unsigned char* end)
    {
        int head[3];
        if (end - p < (long)sizeof(head)) return false;
        std::memcpy(head, p, sizeof(head));
        p += sizeof(head);
        const int n = head[0];
        if (n < 0 || (size_t)(end - p) < (size_t)n * sizeof(Node) || head[1] < kNone || head[1] >= n ||
            head[2] < kNone || head[2] >= n)
            return false;
        nodes_.resize(n);
        if (n > 0) std::memcpy(nodes_.data(), p, n * sizeof(Node));
        p += n * sizeof(Node);
        for (const Node& x : nodes_)
            if (x.parent < kNone || x.parent >= n || x.child1 < kNone || x.child1 >= n || x.child2 < kNone ||
                x.child2 >= n || (x.height > 0 && (x.child1 < 0 || x.child2 < 0)))
                return false;
        root_ = head[1];
        free_ = head[2];
        return true;
    }

private:
    static void Append(std::vector<unsigned char>& out, const void* src, size_t bytes)
    {
        const unsigned char* b = static_cast<const unsigned char*>(src);
        out.insert(out.end(), b, b + bytes);
    }

    struct Node {
        float4 box = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        int parent = kNone;  // the next free node while the node is in the free list
        int child1 = kNone, child2 = kNone;
        int height = -1;     // -1: free
        bool leaf() const { return child1 == kNone; }
    };

    static float Perimeter(float4 b)
    {
        const float wx = b.z - b.x, wy = b.w - b.y;
        return 2.0f * (wx + wy);
    }
    static int Higher(int a, int b) { return a > b ? a : b; }

    // b2DynamicTree::AllocateNode (:56-90): a pool of 16 nodes, doubled when the free list runs out,
    // the new nodes chained in ascending order
    int Allocate()
    {
        if (free_ == kNone) {
            const int old = (int)nodes_.size();
            const int cap = old == 0 ? 16 : 2 * old;
            nodes_.resize(cap);
            for (int i = old; i < cap; ++i) {
                nodes_[i].parent = i + 1 < cap ? i + 1 : kNone;
                nodes_[i].height = -1;
            }
            free_ = old;
        }
        const int id = free_;
        free_ = nodes_[id].parent;
        Node& n = nodes_[id];
        n.parent = kNone;
        n.child1 = kNone;
        n.child2 = kNone;
        n.height = 0;
        return id;
    }
    // b2DynamicTree::FreeNode (:93-100): back on top of the free list
    void Release(int id)
    {
        nodes_[id].parent = free_;
        nodes_[id].height = -1;
        free_ = id;
    }

    void Refit(int i)
    {
        Node& n = nodes_[i];
        n.height = 1 + Higher(nodes_[n.child1].height, nodes_[n.child2].height);
        n.box = Combine(nodes_[n.child1].box, nodes_[n.child2].box);
    }

    // the cost of descending into child c with the leaf's box (b2DynamicTree.cpp:213-239): the new
    // perimeter for a leaf, the perimeter growth for a subtree, plus what the ancestors inherit
    float DescendCost(int c, float4 leafBox, float inherited) const
    {
        const float p = Perimeter(Combine(leafBox, nodes_[c].box));
        if (nodes_[c].leaf()) return p + inherited;
        return (p - Perimeter(nodes_[c].box)) + inherited;
    }

    // b2DynamicTree::InsertLeaf (:179-317): the cheapest sibling by the perimeter heuristic, a new
    // parent over the two, then balance and refit up to the root
    void InsertLeaf(int leaf)
    {
        if (root_ == kNone) {
            root_ = leaf;
            nodes_[leaf].parent = kNone;
            return;
        }
        const float4 leafBox = nodes_[leaf].box;
        int at = root_;
        while (!nodes_[at].leaf()) {
            const float here = Perimeter(nodes_[at].box);
            const float joined = Perimeter(Combine(nodes_[at].box, leafBox));
            const float stop = 2.0f * joined;               // a new parent of this node and the leaf
            const float inherited = 2.0f * (joined - here);  // what every level below adds
            const int c1 = nodes_[at].child1, c2 = nodes_[at].child2;
            const float cost1 = DescendCost(c1, leafBox, inherited);
            const float cost2 = DescendCost(c2, leafBox, inherited);
            if (stop < cost1 && stop < cost2) break;
            at = cost1 < cost2 ? c1 : c2;
        }
        const int sibling = at;
        const int above = nodes_[sibling].parent;
        const int p = Allocate();
        nodes_[p].parent = above;
        nodes_[p].box = Combine(leafBox, nodes_[sibling].box);
        nodes_[p].height = nodes_[sibling].height + 1;
        if (above == kNone) {
            root_ = p;
        } else if (nodes_[above].child1 == sibling) {
            nodes_[above].child1 = p;
        } else {
            nodes_[above].child2 = p;
        }
        nodes_[p].child1 = sibling;
        nodes_[p].child2 = leaf;
        nodes_[sibling].parent = p;
        nodes_[leaf].parent = p;
        for (int i = p; i != kNone; i = nodes_[i].parent) {
            i = Balance(i);
            Refit(i);
        }
    }

    // b2DynamicTree::RemoveLeaf (:319-378): the sibling takes the parent's place, the parent goes
    // back to the pool, the ancestors are balanced and refitted
    void RemoveLeaf(int leaf)
    {
        if (leaf == root_) {
            root_ = kNone;
            return;
        }
        const int p = nodes_[leaf].parent;
        const int gp = nodes_[p].parent;
        const int sibling = nodes_[p].child1 == leaf ? nodes_[p].child2 : nodes_[p].child1;
        if (gp == kNone) {
            root_ = sibling;
            nodes_[sibling].parent = kNone;
            Release(p);
            return;
        }
        if (nodes_[gp].child1 == p) nodes_[gp].child1 = sibling;
        else nodes_[gp].child2 = sibling;
        nodes_[sibling].parent = gp;
        Release(p);
        for (int i = gp; i != kNone; i = nodes_[i].parent) {
            i = Balance(i);
            // the reference refits the box before the height here; both follow from the children
            Refit(i);
        }
    }

    // b2DynamicTree::Balance (:380-520): when one child of node a is more than one level taller, that
    // child rotates up into a's place and a keeps the taller of the child's own children away from it.
    // Returns the node now at a's place.
    int Balance(int a)
    {
        Node& A = nodes_[a];
        if (A.leaf() || A.height < 2) return a;
        const int b = A.child1, c = A.child2;
        const int lean = nodes_[c].height - nodes_[b].height;
        if (lean > 1) return RotateUp(a, c, false);
        if (lean < -1) return RotateUp(a, b, true);
        return a;
    }

    // child `up` of node a (its child1 when leftSide, else child2) takes a's place; a becomes up's
    // child1, and up's lower child replaces `up` under a
    int RotateUp(int a, int up, bool leftSide)
    {
        Node& A = nodes_[a];
        Node& U = nodes_[up];
        const int keep = leftSide ? A.child2 : A.child1;  // a's other child, which stays under a
        const int f = U.child1, g = U.child2;
        U.child1 = a;
        U.parent = A.parent;
        A.parent = up;
        if (U.parent == kNone) {
            root_ = up;
        } else if (nodes_[U.parent].child1 == a) {
            nodes_[U.parent].child1 = up;
        } else {
            nodes_[U.parent].child2 = up;
        }
        // the taller grandchild stays with `up`, the other moves under a
        const bool fTaller = nodes_[f].height > nodes_[g].height;
        const int stay = fTaller ? f : g, move = fTaller ? g : f;
        U.child2 = stay;
        if (leftSide) A.child1 = move;
        else A.child2 = move;
        nodes_[move].parent = a;
        A.box = Combine(nodes_[keep].box, nodes_[move].box);
        U.box = Combine(A.box, nodes_[stay].box);
        A.height = 1 + Higher(nodes_[keep].height, nodes_[move].height);
        U.height = 1 + Higher(A.height, nodes_[stay].height);
        return up;
    }

    std::vector<Node> nodes_;
    int root_ = kNone;
    int free_ = kNone;
};

} // namespace b2g
