// Oracle (test infrastructure only): dynamic AABB tree and broadphase, restated from the reference
// Box2D 2.3.2 Collision/b2DynamicTree.cpp and Collision/b2BroadPhase.{h,cpp}. Node ids double as proxy
// ids, so the free-list allocation order is reproduced exactly, including after proxies are destroyed.
#include "tree.h"

#include <algorithm>

namespace b2o {

Tree::Tree()
{
    capacity = 16;
    nodes.assign(capacity, TreeNode());
    for (int i = 0; i < capacity - 1; ++i) { nodes[i].next = i + 1; nodes[i].height = -1; }
    nodes[capacity - 1].next = kNull;
    nodes[capacity - 1].height = -1;
    freeList = 0;
    nodeCount = 0;
    root = kNull;
}

// b2DynamicTree::AllocateNode (b2DynamicTree.cpp:56-90): capacity doubles when the free list is empty.
int Tree::Allocate()
{
    if (freeList == kNull) {
        capacity *= 2;
        nodes.resize(capacity);
        for (int i = nodeCount; i < capacity - 1; ++i) { nodes[i].next = i + 1; nodes[i].height = -1; }
        nodes[capacity - 1].next = kNull;
        nodes[capacity - 1].height = -1;
        freeList = nodeCount;
    }
    int id = freeList;
    freeList = nodes[id].next;
    nodes[id].parent = kNull;
    nodes[id].child1 = kNull;
    nodes[id].child2 = kNull;
    nodes[id].height = 0;
    nodes[id].user = -1;
    ++nodeCount;
    return id;
}

void Tree::Free(int id)
{
    nodes[id].next = freeList;
    nodes[id].height = -1;
    freeList = id;
    --nodeCount;
}

int Tree::CreateProxy(const AABB& aabb, int user)
{
    int id = Allocate();
    Vec2 r = V(kAabbExtension, kAabbExtension);
    nodes[id].aabb.lo = aabb.lo - r;
    nodes[id].aabb.hi = aabb.hi + r;
    nodes[id].user = user;
    nodes[id].height = 0;
    InsertLeaf(id);
    return id;
}

void Tree::DestroyProxy(int id)
{
    RemoveLeaf(id);
    Free(id);
}

// b2DynamicTree::MoveProxy (b2DynamicTree.cpp:133-177): refatten by the extension and 2x displacement.
bool Tree::MoveProxy(int id, const AABB& aabb, Vec2 displacement)
{
    if (Contains(nodes[id].aabb, aabb)) return false;
    RemoveLeaf(id);
    AABB b = aabb;
    Vec2 r = V(kAabbExtension, kAabbExtension);
    b.lo = b.lo - r;
    b.hi = b.hi + r;
    Vec2 d = kAabbMultiplier * displacement;
    if (d.x < 0.0f) b.lo.x += d.x; else b.hi.x += d.x;
    if (d.y < 0.0f) b.lo.y += d.y; else b.hi.y += d.y;
    nodes[id].aabb = b;
    InsertLeaf(id);
    return true;
}

// b2DynamicTree::InsertLeaf (b2DynamicTree.cpp:179-317): perimeter-cost descent, then refit upward.
void Tree::InsertLeaf(int leaf)
{
    if (root == kNull) { root = leaf; nodes[root].parent = kNull; return; }
    AABB leafAABB = nodes[leaf].aabb;
    int index = root;
    while (!nodes[index].IsLeaf()) {
        int child1 = nodes[index].child1, child2 = nodes[index].child2;
        float area = Perimeter(nodes[index].aabb);
        AABB combined = Combine(nodes[index].aabb, leafAABB);
        float combinedArea = Perimeter(combined);
        float cost = 2.0f * combinedArea;
        float inheritanceCost = 2.0f * (combinedArea - area);
        float cost1, cost2;
        {
            AABB a = Combine(leafAABB, nodes[child1].aabb);
            if (nodes[child1].IsLeaf()) cost1 = Perimeter(a) + inheritanceCost;
            else cost1 = (Perimeter(a) - Perimeter(nodes[child1].aabb)) + inheritanceCost;
        }
        {
            AABB a = Combine(leafAABB, nodes[child2].aabb);
            if (nodes[child2].IsLeaf()) cost2 = Perimeter(a) + inheritanceCost;
            else cost2 = (Perimeter(a) - Perimeter(nodes[child2].aabb)) + inheritanceCost;
        }
        if (cost < cost1 && cost < cost2) break;
        index = cost1 < cost2 ? child1 : child2;
    }
    int sibling = index;
    int oldParent = nodes[sibling].parent;
    int newParent = Allocate();
    nodes[newParent].parent = oldParent;
    nodes[newParent].user = -1;
    nodes[newParent].aabb = Combine(leafAABB, nodes[sibling].aabb);
    nodes[newParent].height = nodes[sibling].height + 1;
    if (oldParent != kNull) {
        if (nodes[oldParent].child1 == sibling) nodes[oldParent].child1 = newParent;
        else nodes[oldParent].child2 = newParent;
    } else {
        root = newParent;
    }
    nodes[newParent].child1 = sibling;
    nodes[newParent].child2 = leaf;
    nodes[sibling].parent = newParent;
    nodes[leaf].parent = newParent;
    index = nodes[leaf].parent;
    while (index != kNull) {
        index = Balance(index);
        int c1 = nodes[index].child1, c2 = nodes[index].child2;
        nodes[index].height = 1 + Max(nodes[c1].height, nodes[c2].height);
        nodes[index].aabb = Combine(nodes[c1].aabb, nodes[c2].aabb);
        index = nodes[index].parent;
    }
}

// b2DynamicTree::RemoveLeaf (b2DynamicTree.cpp:319-378)
void Tree::RemoveLeaf(int leaf)
{
    if (leaf == root) { root = kNull; return; }
    int parent = nodes[leaf].parent;
    int grandParent = nodes[parent].parent;
    int sibling = nodes[parent].child1 == leaf ? nodes[parent].child2 : nodes[parent].child1;
    if (grandParent != kNull) {
        if (nodes[grandParent].child1 == parent) nodes[grandParent].child1 = sibling;
        else nodes[grandParent].child2 = sibling;
        nodes[sibling].parent = grandParent;
        Free(parent);
        int index = grandParent;
        while (index != kNull) {
            index = Balance(index);
            int c1 = nodes[index].child1, c2 = nodes[index].child2;
            nodes[index].aabb = Combine(nodes[c1].aabb, nodes[c2].aabb);
            nodes[index].height = 1 + Max(nodes[c1].height, nodes[c2].height);
            index = nodes[index].parent;
        }
    } else {
        root = sibling;
        nodes[sibling].parent = kNull;
        Free(parent);
    }
}

// b2DynamicTree::Balance (b2DynamicTree.cpp:380-520): single left or right rotation.
int Tree::Balance(int iA)
{
    TreeNode* A = &nodes[iA];
    if (A->IsLeaf() || A->height < 2) return iA;
    int iB = A->child1, iC = A->child2;
    TreeNode* B = &nodes[iB];
    TreeNode* C = &nodes[iC];
    int balance = C->height - B->height;
    if (balance > 1) {
        int iF = C->child1, iG = C->child2;
        TreeNode* F = &nodes[iF];
        TreeNode* G = &nodes[iG];
        C->child1 = iA;
        C->parent = A->parent;
        A->parent = iC;
        if (C->parent != kNull) {
            if (nodes[C->parent].child1 == iA) nodes[C->parent].child1 = iC;
            else nodes[C->parent].child2 = iC;
        } else {
            root = iC;
        }
        if (F->height > G->height) {
            C->child2 = iF; A->child2 = iG; G->parent = iA;
            A->aabb = Combine(B->aabb, G->aabb);
            C->aabb = Combine(A->aabb, F->aabb);
            A->height = 1 + Max(B->height, G->height);
            C->height = 1 + Max(A->height, F->height);
        } else {
            C->child2 = iG; A->child2 = iF; F->parent = iA;
            A->aabb = Combine(B->aabb, F->aabb);
            C->aabb = Combine(A->aabb, G->aabb);
            A->height = 1 + Max(B->height, F->height);
            C->height = 1 + Max(A->height, G->height);
        }
        return iC;
    }
    if (balance < -1) {
        int iD = B->child1, iE = B->child2;
        TreeNode* D = &nodes[iD];
        TreeNode* E = &nodes[iE];
        B->child1 = iA;
        B->parent = A->parent;
        A->parent = iB;
        if (B->parent != kNull) {
            if (nodes[B->parent].child1 == iA) nodes[B->parent].child1 = iB;
            else nodes[B->parent].child2 = iB;
        } else {
            root = iB;
        }
        if (D->height > E->height) {
            B->child2 = iD; A->child1 = iE; E->parent = iA;
            A->aabb = Combine(C->aabb, E->aabb);
            B->aabb = Combine(A->aabb, D->aabb);
            A->height = 1 + Max(C->height, E->height);
            B->height = 1 + Max(A->height, D->height);
        } else {
            B->child2 = iE; A->child1 = iD; D->parent = iA;
            A->aabb = Combine(C->aabb, D->aabb);
            B->aabb = Combine(A->aabb, E->aabb);
            A->height = 1 + Max(C->height, D->height);
            B->height = 1 + Max(A->height, E->height);
        }
        return iB;
    }
    return iA;
}

int Tree::Height() const { return root == kNull ? 0 : nodes[root].height; }

// b2DynamicTree::GetMaxBalance (b2DynamicTree.cpp:675-697): the largest child height difference of
// the internal nodes, over the whole node pool.
int Tree::MaxBalance() const
{
    int best = 0;
    for (int i = 0; i < capacity; ++i) {
        const TreeNode& n = nodes[i];
        if (n.height <= 1) continue;
        const int d = nodes[n.child2].height - nodes[n.child1].height;
        best = Max(best, d < 0 ? -d : d);
    }
    return best;
}

// b2DynamicTree::GetAreaRatio (b2DynamicTree.cpp:534-559): the perimeters of every allocated node,
// summed in pool order, over the root's.
float Tree::AreaRatio() const
{
    if (root == kNull) return 0.0f;
    const float rootArea = Perimeter(nodes[root].aabb);
    float total = 0.0f;
    for (int i = 0; i < capacity; ++i)
        if (nodes[i].height >= 0) total += Perimeter(nodes[i].aabb);
    return total / rootArea;
}

// ---------------------------------------------------------------- broadphase
int BroadPhase::CreateProxy(const AABB& aabb, int user)
{
    int id = tree.CreateProxy(aabb, user);
    ++proxyCount;
    moveBuffer.push_back(id);
    return id;
}

void BroadPhase::DestroyProxy(int id)
{
    for (int& m : moveBuffer) if (m == id) m = kNull;
    --proxyCount;
    tree.DestroyProxy(id);
}

void BroadPhase::MoveProxy(int id, const AABB& aabb, Vec2 displacement)
{
    if (tree.MoveProxy(id, aabb, displacement)) moveBuffer.push_back(id);
}

void BroadPhase::TouchProxy(int id) { moveBuffer.push_back(id); }

// b2BroadPhase::UpdatePairs (b2BroadPhase.h:188-241): query every moved proxy's fat AABB, record
// (min, max) proxy-id pairs, sort lexicographically and drop duplicates. The resulting ordered list is
// what the contact manager consumes.
void BroadPhase::ComputePairs(std::vector<Pair>& out)
{
    pairs.clear();
    std::vector<int> stack;
    for (int q : moveBuffer) {
        if (q == kNull) continue;
        const AABB fat = tree.nodes[q].aabb;
        stack.clear();
        if (tree.root != kNull) stack.push_back(tree.root);
        while (!stack.empty()) {
            int node = stack.back();
            stack.pop_back();
            if (node == kNull) continue;
            const TreeNode& n = tree.nodes[node];
            if (!Overlap(n.aabb, fat)) continue;
            if (n.IsLeaf()) {
                if (node != q) pairs.push_back(Pair{Min(node, q), Max(node, q)});
            } else {
                stack.push_back(n.child1);
                stack.push_back(n.child2);
            }
        }
    }
    moveBuffer.clear();
    std::sort(pairs.begin(), pairs.end(), [](const Pair& a, const Pair& b) {
        return a.a < b.a || (a.a == b.a && a.b < b.b);
    });
    out.clear();
    for (size_t i = 0; i < pairs.size(); ) {
        out.push_back(pairs[i]);
        size_t j = i + 1;
        while (j < pairs.size() && pairs[j].a == pairs[i].a && pairs[j].b == pairs[i].b) ++j;
        i = j;
    }
}

} // namespace b2o
