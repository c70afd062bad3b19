// Oracle (test infrastructure only): dynamic AABB tree and broadphase declarations.
#pragma once
#include "b2o.h"

namespace b2o {

constexpr int kNull = -1;

struct TreeNode {
    AABB aabb{};
    int user = -1;
    int parent = kNull; // doubles as the free-list link ("next") while the node is free
    int child1 = kNull, child2 = kNull;
    int height = -1;
    int next = kNull;
    bool IsLeaf() const { return child1 == kNull; }
};

struct Tree {
    std::vector<TreeNode> nodes;
    int root, freeList, nodeCount, capacity;
    Tree();
    int Allocate();
    void Free(int id);
    int CreateProxy(const AABB& aabb, int user);
    void DestroyProxy(int id);
    bool MoveProxy(int id, const AABB& aabb, Vec2 displacement);
    void InsertLeaf(int leaf);
    void RemoveLeaf(int leaf);
    int Balance(int iA);
    int Height() const;
    int MaxBalance() const;
    float AreaRatio() const;
};

struct Pair { int a, b; };

struct BroadPhase {
    Tree tree;
    int proxyCount = 0;
    std::vector<int> moveBuffer;
    std::vector<Pair> pairs;
    int CreateProxy(const AABB& aabb, int user);
    void DestroyProxy(int id);
    void MoveProxy(int id, const AABB& aabb, Vec2 displacement);
    void TouchProxy(int id);
    bool TestOverlap(int a, int b) const { return Overlap(tree.nodes[a].aabb, tree.nodes[b].aabb); }
    const AABB& FatAABB(int id) const { return tree.nodes[id].aabb; }
    void ComputePairs(std::vector<Pair>& out);
};

} // namespace b2o
