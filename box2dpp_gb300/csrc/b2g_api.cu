// Host runtime of the GB300 Box2D step and the C-ABI declared in include/box2d_gb300.h.
//
// The host keeps a mirror of each world's bodies, fixtures, proxies and joints. Creation calls
// (b2World::CreateBody, b2Body::CreateFixture, b2World::CreateJoint) run their setup arithmetic here,
// exactly as the reference does on its host: polygon hulls, mass data, initial transforms and AABBs,
// proxy ids. The mirror is uploaded once into device columns (b2g_world.h); from then on every step
// runs on the device and the host only reads state back when asked. A creation call after steps
// first pulls the device state back, so the mirror stays authoritative for the next upload.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <numeric>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/box2d_gb300.h"
#include "b2g_tree.h"
#include "b2g_world.h"

cudaError_t b2gLaunchNarrowphase(const b2g::Batch& B, const int4* chunks, int n, cudaStream_t stream);
cudaError_t b2gLaunchStep(const b2g::Batch& B, const b2g::StepParams& P, const int* schedule, int first, int count,
                          int threads, int smemRows, int smemContacts, cudaStream_t stream);
cudaError_t b2gLaunchToi(const b2g::Batch& B, const b2g::StepParams& P, const int4* chunks, int n, cudaStream_t stream);
cudaError_t b2gLaunchBodyEdits(const b2g::Batch& B, const b2g::BodyEdit* edits, int n, cudaStream_t stream);
cudaError_t b2gLaunchContactEdits(const b2g::Batch& B, const b2g::ContactEdit* edits, int n, cudaStream_t stream);
cudaError_t b2gLaunchStepToi(const b2g::Batch& B, const b2g::StepParams& P, const int* schedule, int first, int count,
                             int threads, int smemRows, int smemContacts, cudaStream_t stream);
cudaError_t b2gLaunchSinCos(const float* x, float* s, float* c, int n, cudaStream_t stream);
b2g::MlpView b2gMlpView(const gb_mlp* m);
cudaError_t b2gLaunchQueryAabb(const b2g::Batch& B, int w, const float4* boxes, int n, const int* offsets, int* counts,
                               int* fill, int cap, cudaStream_t stream);
cudaError_t b2gLaunchRayCast(const b2g::Batch& B, int w, const float4* rays, int n, int* fixture, float* hit,
                             cudaStream_t stream);
cudaError_t b2gLaunchRayCastAll(const b2g::Batch& B, int w, int fixCount, float4 ray, float4* hits, int* count, int cap,
                                cudaStream_t stream);
cudaError_t b2gLaunchCollide(int n, const b2g::Shape* a, const float4* xa, const b2g::Shape* b, const float4* xb,
                             int4* oi, float4* of, cudaStream_t stream);

using namespace b2g;

namespace {

struct HBody {
    int type = kStatic, flags = 0;
    Xf xf{};
    Sweep sw{};
    Vec2 v{0, 0};
    float w = 0;
    Vec2 force{0, 0};
    float torque = 0;
    float mass = 0, invMass = 0, I = 0, invI = 0;
    float linDamp = 0, angDamp = 0, gravScale = 1, sleepTime = 0;
    int fixtureList = kNullIdx, contactList = kNullIdx, jointList = kNullIdx, next = kNullIdx;
    bool alive = true; // false once destroyed: its columns are zeros and it is in no list
};

struct HFixture {
    int body = kNullIdx, next = kNullIdx;
    Shape shape{};
    float density = 0, friction = 0.2f, restitution = 0;
    int category = 1, mask = 0xFFFF, group = 0, sensor = 0;
    int proxyId = kNullIdx;
    float4 aabb{};
};

struct HContacts { // device contact columns of one world, pulled back before a host-side change
    std::vector<int4> ci, ce, mh;
    std::vector<float4> cp, mv, mp0, mp1;
    std::vector<int> order, cnext;
};

struct HWorld {
    gb_world_def def{};
    bool autoClear = true;  // b2World::SetAutoClearForces
    int bodyList = kNullIdx, jointList = kNullIdx;
    std::vector<HBody> bodies;
    std::vector<HFixture> fixtures;
    std::vector<Joint> joints;
    std::vector<float4> fat;
    std::vector<int> pfix, moved;
    // The reference tree's node ids (b2DynamicTree): never-used ids are handed out in order from
    // nodeFresh; freed ids are reused last-in first-out. nodeFree holds the freed ids, -1 standing for
    // an internal node (a leaf's parent) whose id is never needed: a freed leaf is always on top of
    // its parent, and a proxy takes a leaf and then a parent, so leaves only ever come back as leaves.
    int nodeFresh = 0, proxyCount = 0;
    std::vector<int> nodeFree;
    bool treeLost = false; // a leaf would have taken an internal node's id (never expected)
    // the reference tree's shape, kept only when the handle tracks trees (gb_world_track_tree):
    // treeIncomplete when the device's tree log ran out of room or an id disagreed with nodeFresh
    bool trackTree = false, treeIncomplete = false;
    ProxyTree tree;
    int newFixture = 0;
    int capHint = 0;  // contact slots the next upload gives at least (grown after an overflow)
    WorldState state{};
    bool hasState = false; // state/contacts valid (pulled back from, or never sent to, the device)
    HContacts contacts;
};

template <typename T> struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
};

// One launch of the step over a contiguous range of the schedule (worlds sorted largest first).
struct LaunchClass {
    int first, count, threads, rows, contacts;
};
using LaunchPlan = std::vector<LaunchClass>;
constexpr int kMaxClasses = 4;

} // namespace

struct gb_world {
    std::vector<HWorld> worlds;
    std::vector<WorldDesc> desc;
    Batch batch{};
    std::vector<void*> allocations;
    std::vector<size_t> allocationBytes;  // sizes of allocations (the filtered step's snapshot)
    // user contact filter (gb_world_set_contact_filter): the callback, the device verdict table,
    // and a copy of every device column taken before each step so that a step can be run again
    gb_should_collide_fn filterFn = nullptr;
    void* filterUser = nullptr;
    unsigned long long* dFilterKeys = nullptr;
    int* dFilterVals = nullptr;
    int* dFilterMiss = nullptr;
    int filterCap = 0, filterUsed = 0;
    std::vector<void*> shadow;
    // grow-and-retry (gb_world_set_recovery): attempts per step, a copy of every device column taken
    // before each step, and the steps that were run again
    int recoverAttempts = 0;
    std::vector<void*> recoverShadow;
    long long recoveries = 0;
    long long filterReplays = 0;
    int* dSchedule = nullptr;
    // row chunks of the flat pre-passes in schedule order (see kRowChunk), and the first chunk of
    // each schedule slot (one entry more: the total)
    int4* dNpChunks = nullptr;
    int4* dToiChunks = nullptr;
    std::vector<int> npChunkStart, toiChunkStart;
    cudaStream_t stream = nullptr;
    bool ownStream = false;
    bool onDevice = false;   // device columns hold the current state
    bool hostDirty = true;   // host mirror has changes not yet uploaded
    bool locked = false;
    // launch plan: size classes of worlds, each a launch with its own CTA size and shared memory
    std::vector<int> schedule;      // world indices, largest first
    std::vector<int> scheduleSize;  // body count of schedule[i]
    LaunchPlan plan;
    cudaStream_t side[kMaxClasses] = {};
    cudaEvent_t fork = nullptr, join[kMaxClasses] = {};
    // the step's per-class pipelines: class i on pipe[i], priorities falling with i
    cudaStream_t pipe[kMaxClasses] = {};
    cudaEvent_t pipeJoin[kMaxClasses] = {};
    // online autotuning of the plan over real steps (every plan gives identical results)
    std::vector<LaunchPlan> candidates;
    std::vector<float> candidateMs;
    std::vector<cudaEvent_t> tuneEvents;
    int tuneSteps = 0, tuneIndex = -1, tuneRep = 0;
    // one captured step (every launch of the plan) replayed by gb_world_graph_step
    cudaGraphExec_t graph = nullptr;
    float graphDt = 0.0f;
    int graphVi = -1, graphPi = -1, graphSolver = -1, graphMeasure = -1, graphWarm = -1;
    const float* graphLog = nullptr;
    float graphTol = -1.0f;
    LaunchPlan graphPlan;
    int solver = kSolverPlain;
    int contactCapLimit = 0;    // > 0: contact slots per world at the first upload (gb_world_set_limits)
    int maxToiEvents = 4096;    // time-of-impact events per world per step
    float tolerance = 0.0f;
    int measureResidual = 0;
    int warmMode = kWarmReference;
    bool eventsEnabled = false;
    bool treeTrack = false;  // every world keeps its tree (gb_world_track_tree); the device logs moves
    MlpView mlp{};
    BodyEdit* dEdits = nullptr;  // device copy of the last gb_body_edits call
    int editCap = 0;
    ContactEdit* dContactEdits = nullptr;  // device copy of the last gb_contact_edits call
    int contactEditCap = 0;
    bool splitOpen = false;  // gb_world_step_begin ran, gb_world_step_end not yet
    float splitDt = 0.0f;
    int splitVi = 0, splitPi = 0;
    float* logX = nullptr;   // contact-point log (device), see gb_world_set_contact_log
    float* logT = nullptr;
    int* logCount = nullptr;
    int logCap = 0;
    // pipelined transfers (gb_set_forces_async, gb_get_transforms_async): an upload and a download
    // stream, two device staging buffers per direction used in turn, and the events that order them
    // against the handle's stream
    cudaStream_t upStream = nullptr, downStream = nullptr;
    float4* forceStage[2] = {};
    float4* xfStage[2] = {};
    size_t stageBodies = 0;
    cudaEvent_t upDone[2] = {}, forceTaken[2] = {}, xfReady[2] = {}, downDone[2] = {};
    unsigned upCount = 0, downCount = 0;
};

namespace {

inline int __float_as_int_host(float f)
{
    int i;
    std::memcpy(&i, &f, sizeof(i));
    return i;
}

gb_status cudaErr(cudaError_t e)
{
    if (e == cudaSuccess) return GB_OK;
    std::fprintf(stderr, "box2d_gb300: CUDA error: %s\n", cudaGetErrorString(e));
    return GB_ERR_CUDA;
}

#define GB_CUDA(x)                                   \
    do {                                             \
        gb_status s_ = cudaErr(x);                   \
        if (s_ != GB_OK) return s_;                  \
    } while (0)

// b2Body::ResetMassData (Box2D/Dynamics/b2Body.cpp:283-352)
void ResetMassData(HWorld& W, int bi)
{
    HBody& b = W.bodies[bi];
    b.mass = 0.0f; b.invMass = 0.0f; b.I = 0.0f; b.invI = 0.0f;
    b.sw.localCenter = V(0.0f, 0.0f);
    if (b.type == kStatic || b.type == kKinematic) {
        b.sw.c0 = b.xf.p;
        b.sw.c = b.xf.p;
        b.sw.a0 = b.sw.a;
        return;
    }
    Vec2 localCenter = V(0.0f, 0.0f);
    for (int f = b.fixtureList; f != kNullIdx; f = W.fixtures[f].next) {
        const HFixture& fx = W.fixtures[f];
        if (fx.density == 0.0f) continue;
        MassData md;
        ComputeMass(fx.shape, fx.density, &md);
        b.mass += md.mass;
        localCenter = localCenter + md.mass * md.center;
        b.I += md.I;
    }
    if (b.mass > 0.0f) {
        b.invMass = 1.0f / b.mass;
        localCenter.x *= b.invMass;
        localCenter.y *= b.invMass;
    } else {
        b.mass = 1.0f;
        b.invMass = 1.0f;
    }
    if (b.I > 0.0f && (b.flags & kBFixedRot) == 0) {
        b.I -= b.mass * Dot(localCenter, localCenter);
        b.invI = 1.0f / b.I;
    } else {
        b.I = 0.0f;
        b.invI = 0.0f;
    }
    Vec2 oldCenter = b.sw.c;
    b.sw.localCenter = localCenter;
    b.sw.c = Mul(b.xf, b.sw.localCenter);
    b.sw.c0 = b.sw.c;
    b.v = b.v + Cross(b.w, b.sw.c - oldCenter);
}

// Proxy ids are node ids of the reference's b2DynamicTree. b2DynamicTree::CreateProxy takes a node
// for the leaf, and InsertLeaf one more for its new parent unless the tree was empty
// (b2DynamicTree.cpp:56-131, 179-194); DestroyProxy's RemoveLeaf frees the leaf's parent unless the
// leaf was the root, then the leaf itself (:124-130, 319-377); MoveProxy frees one internal node and
// takes it straight back (LIFO), and Balance moves no ids. The free list is therefore a stack of
// (parent, leaf) pairs over the never-used ids, and the next leaf id follows without the tree's shape.
int AllocNode(HWorld& W, bool leaf)
{
    if (!W.nodeFree.empty()) {
        const int id = W.nodeFree.back();
        W.nodeFree.pop_back();
        if (leaf && id < 0) W.treeLost = true;
        return id;
    }
    return W.nodeFresh++;
}

int AllocateProxy(HWorld& W, float4 fatAabb, int fixture)
{
    int id = AllocNode(W, true);
    if (W.proxyCount > 0) AllocNode(W, false);
    ++W.proxyCount;
    if (id < 0) id = W.nodeFresh++;  // unreachable by the pairing above; keeps the id valid
    if ((int)W.fat.size() <= id) {
        W.fat.resize(id + 1, make_float4(0, 0, 0, 0));
        W.pfix.resize(id + 1, kNullIdx);
        W.moved.resize(id + 1, 0);
    }
    W.fat[id] = fatAabb;
    W.pfix[id] = fixture;
    W.moved[id] = 1;
    if (W.trackTree && W.tree.Insert(fatAabb) != id) W.treeIncomplete = true;
    return id;
}

// b2BroadPhase::DestroyProxy (Collision/b2BroadPhase.cpp:74-79): out of the move buffer, the leaf's
// parent (when the tree has more leaves) and then the leaf back to the free list.
void FreeProxy(HWorld& W, int id)
{
    if (W.proxyCount > 1) W.nodeFree.push_back(-1);
    W.nodeFree.push_back(id);
    --W.proxyCount;
    if (W.trackTree) W.tree.Remove(id);
    W.fat[id] = make_float4(0, 0, 0, 0);
    W.pfix[id] = kNullIdx;
    W.moved[id] = 0;
}

Shape MakeShape(int type, const float* s, int n)
{
    Shape sh;
    std::memset(&sh, 0, sizeof(sh));
    switch (type) {
    case 0:
        sh.type = kCircle; sh.count = 1; sh.v[0] = V(s[0], s[1]); sh.radius = s[2];
        break;
    case 1:
        sh.type = kEdge; sh.count = 2; sh.radius = kPolygonRadius;
        sh.v[0] = V(s[0], s[1]); sh.v[1] = V(s[2], s[3]); sh.v[2] = V(s[4], s[5]); sh.v[3] = V(s[6], s[7]);
        sh.hasV0 = s[8] != 0.0f; sh.hasV3 = s[9] != 0.0f;
        sh.chain = (int)s[10];
        break;
    case 2: {
        Vec2 pts[kMaxPolyVerts];
        int m = std::min(n, kMaxPolyVerts);
        for (int i = 0; i < m; ++i) pts[i] = V(s[2 * i], s[2 * i + 1]);
        PolygonSet(sh, pts, n);
        break;
    }
    default:
        if (n == 5) PolygonSetAsBox(sh, s[0], s[1], V(s[2], s[3]), s[4]);
        else PolygonSetAsBox(sh, s[0], s[1]);
        break;
    }
    return sh;
}

template <typename T> gb_status DevAlloc(gb_world* g, T** p, size_t n)
{
    *p = nullptr;
    if (n == 0) n = 1;
    void* ptr = nullptr;
    GB_CUDA(cudaMalloc(&ptr, n * sizeof(T)));
    g->allocations.push_back(ptr);
    g->allocationBytes.push_back(n * sizeof(T));
    *p = static_cast<T*>(ptr);
    return GB_OK;
}

void FreeDevice(gb_world* g)
{
    // a captured step holds the device addresses being freed
    if (g->graph) cudaGraphExecDestroy(g->graph);
    g->graph = nullptr;
    for (void* p : g->allocations) cudaFree(p);
    g->allocations.clear();
    g->allocationBytes.clear();
    for (void* p : g->shadow) cudaFree(p);
    g->shadow.clear();
    for (void* p : g->recoverShadow) cudaFree(p);
    g->recoverShadow.clear();
    std::memset(&g->batch, 0, sizeof(g->batch));
    g->dSchedule = nullptr;
    g->dNpChunks = g->dToiChunks = nullptr;
    g->npChunkStart.clear();
    g->toiChunkStart.clear();
}

int NextPow2(int x)
{
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Pull the device state of every world back into the host mirror.
// The device's tree log replayed into each world's host tree (gb_world_track_tree), its count cleared
// on the device. Records go in log order, except that each step's discrete-phase records, written by
// many threads at once, are first put in the reference's order: the world's body list (newest body
// first), then each body's fixture list (b2World::Solve, Dynamics/b2World.cpp:494-514). The caller has
// synchronised the world's streams.
gb_status DrainTreeLog(gb_world* g)
{
    if (!g->treeTrack || !g->onDevice || !g->batch.treeLogId) return GB_OK;
    const int nw = (int)g->worlds.size();
    std::vector<WorldState> st(nw);
    GB_CUDA(cudaMemcpy(st.data(), g->batch.state, nw * sizeof(WorldState), cudaMemcpyDeviceToHost));
    std::vector<int> ids, rank, run;
    std::vector<float4> fats;
    for (int wi = 0; wi < nw; ++wi) {
        const int n = st[wi].treeLogCount;
        if (n == 0) continue;
        HWorld& W = g->worlds[wi];
        const WorldDesc& d = g->desc[wi];
        const int cap = kTreeLogPerProxy * d.proxyCap + kTreeLogExtra;
        const size_t at = (size_t)kTreeLogPerProxy * d.proxyBase + (size_t)kTreeLogExtra * wi;
        const int zero = 0;
        GB_CUDA(cudaMemcpy(&g->batch.state[wi].treeLogCount, &zero, sizeof(int), cudaMemcpyHostToDevice));
        if (n > cap) {
            W.treeIncomplete = true;
            continue;
        }
        ids.resize(n);
        fats.resize(n);
        GB_CUDA(cudaMemcpy(ids.data(), g->batch.treeLogId + at, n * sizeof(int), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(fats.data(), g->batch.treeLogFat + at, n * sizeof(float4), cudaMemcpyDeviceToHost));
        rank.assign(d.proxyCap, d.proxyCap);
        int r = 0;
        for (int b = W.bodyList; b != kNullIdx; b = W.bodies[b].next)
            for (int f = W.bodies[b].fixtureList; f != kNullIdx; f = W.fixtures[f].next)
                if (W.fixtures[f].proxyId != kNullIdx) rank[W.fixtures[f].proxyId] = r++;
        for (int k = 0; k < n;) {
            const int kind = ids[k] & 3, pid = ids[k] >> 2;
            if (pid < 0 || pid >= d.proxyCap) {
                W.treeIncomplete = true;
                break;
            }
            if (kind != kTreeDiscrete) {
                if (kind == kTreeOrdered) W.tree.Move(pid, fats[k]);
                ++k;
                continue;
            }
            int e = k;
            while (e < n && (ids[e] & 3) == kTreeDiscrete) ++e;
            run.resize(e - k);
            std::iota(run.begin(), run.end(), k);
            std::sort(run.begin(), run.end(), [&](int a, int b) { return rank[ids[a] >> 2] < rank[ids[b] >> 2]; });
            for (int i : run) W.tree.Move(ids[i] >> 2, fats[i]);
            k = e;
        }
    }
    return GB_OK;
}

// Before a step of a handle that tracks trees: the previous step's tree log is replayed first.
gb_status TreeSync(gb_world* g)
{
    if (!g->treeTrack || !g->onDevice) return GB_OK;
    GB_CUDA(cudaStreamSynchronize(g->stream));
    return DrainTreeLog(g);
}

gb_status Download(gb_world* g)
{
    if (!g->onDevice) return GB_OK;
    GB_CUDA(cudaStreamSynchronize(g->stream));
    {
        gb_status s = DrainTreeLog(g);
        if (s != GB_OK) return s;
    }
    const Batch& B = g->batch;
    for (size_t wi = 0; wi < g->worlds.size(); ++wi) {
        HWorld& W = g->worlds[wi];
        const WorldDesc& d = g->desc[wi];
        int nb = d.bodyCount, nf = d.fixCount, np = d.proxyCap, nc = d.contactCap;
        std::vector<float4> xf(nb), sw(nb), sw0(nb), vel(nb), frc(nb);
        std::vector<int4> bi(nb), bj(nb);
        GB_CUDA(cudaMemcpy(xf.data(), B.xf + d.bodyBase, nb * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(sw.data(), B.sw + d.bodyBase, nb * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(sw0.data(), B.sw0 + d.bodyBase, nb * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(vel.data(), B.vel + d.bodyBase, nb * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(frc.data(), B.frc + d.bodyBase, nb * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(bi.data(), B.bi + d.bodyBase, nb * sizeof(int4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(bj.data(), B.bj + d.bodyBase, nb * sizeof(int4), cudaMemcpyDeviceToHost));
        for (int i = 0; i < nb; ++i) {
            HBody& b = W.bodies[i];
            b.xf.p = V(xf[i].x, xf[i].y); b.xf.q.s = xf[i].z; b.xf.q.c = xf[i].w;
            b.sw.c = V(sw[i].x, sw[i].y); b.sw.a = sw[i].z; b.sw.alpha0 = sw[i].w;
            b.sw.c0 = V(sw0[i].x, sw0[i].y); b.sw.a0 = sw0[i].z; b.sleepTime = sw0[i].w;
            b.v = V(vel[i].x, vel[i].y); b.w = vel[i].z;
            b.force = V(frc[i].x, frc[i].y); b.torque = frc[i].z;
            b.flags = bi[i].y; b.contactList = bi[i].w;
        }
        std::vector<float4> faabb(nf);
        GB_CUDA(cudaMemcpy(faabb.data(), B.faabb + d.fixBase, nf * sizeof(float4), cudaMemcpyDeviceToHost));
        for (int i = 0; i < nf; ++i) W.fixtures[i].aabb = faabb[i];
        W.fat.resize(np); W.moved.resize(np);
        GB_CUDA(cudaMemcpy(W.fat.data(), B.fat + d.proxyBase, np * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(W.moved.data(), B.moved + d.proxyBase, np * sizeof(int), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(&W.state, B.state + wi, sizeof(WorldState), cudaMemcpyDeviceToHost));
        HContacts& C = W.contacts;
        C.ci.resize(nc); C.ce.resize(nc); C.mh.resize(nc); C.cp.resize(nc); C.mv.resize(nc); C.mp0.resize(nc);
        C.mp1.resize(nc); C.order.resize(nc); C.cnext.resize(nc);
        GB_CUDA(cudaMemcpy(C.ci.data(), B.ci + d.contactBase, nc * sizeof(int4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(C.ce.data(), B.ce + d.contactBase, nc * sizeof(int4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(C.mh.data(), B.mh + d.contactBase, nc * sizeof(int4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(C.cp.data(), B.cp + d.contactBase, nc * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(C.mv.data(), B.mv + d.contactBase, nc * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(C.mp0.data(), B.mp0 + d.contactBase, nc * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(C.mp1.data(), B.mp1 + d.contactBase, nc * sizeof(float4), cudaMemcpyDeviceToHost));
        {
            // the contact list (orderStart of the state read above)
            std::fill(C.order.begin(), C.order.end(), 0);
            const int live = std::min(W.state.contactCount, nc);
            if (live > 0)
                GB_CUDA(cudaMemcpy(C.order.data(), B.order + 2 * (size_t)d.contactBase + W.state.orderStart,
                                   live * sizeof(int), cudaMemcpyDeviceToHost));
        }
        GB_CUDA(cudaMemcpy(C.cnext.data(), B.cnext + d.contactBase, nc * sizeof(int), cudaMemcpyDeviceToHost));
        if (d.jointCount > 0)
            GB_CUDA(cudaMemcpy(W.joints.data(), B.joint + d.jointBase, d.jointCount * sizeof(Joint), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(&W.state, B.state + wi, sizeof(WorldState), cudaMemcpyDeviceToHost));
        W.newFixture = W.state.newFixture;
        W.hasState = true;
    }
    g->onDevice = false;
    return GB_OK;
}

template <typename T> gb_status Put(T* dst, const std::vector<T>& src, size_t n)
{
    if (n == 0) return GB_OK;
    GB_CUDA(cudaMemcpy(dst, src.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    return GB_OK;
}

// ------------------------------------------------------------------ launch plans
int RoundUp(int x, int m) { return (x + m - 1) / m * m; }

// A class over schedule[first, first + count): shared memory sized for its largest world (island rows
// ~ bodies plus the static bodies repeated per island, contacts ~ 2.5 per body), within 36 KB.
LaunchClass MakeClass(const gb_world* g, int first, int count, int threads)
{
    int maxBodies = 0;
    for (int i = first; i < first + count; ++i) maxBodies = std::max(maxBodies, g->scheduleSize[i]);
    LaunchClass c;
    c.first = first;
    c.count = count;
    c.threads = threads;
    c.rows = std::min(640, std::max(64, RoundUp(maxBodies + maxBodies / 4 + 16, 32)));
    c.contacts = std::min(1024, std::max(128, RoundUp(maxBodies * 5 / 2 + 32, 32)));
    return c;
}

// Split the schedule (largest first) at body-count thresholds (descending); one CTA size per class.
LaunchPlan SplitPlan(const gb_world* g, const std::vector<int>& thresholds, const std::vector<int>& threads)
{
    LaunchPlan plan;
    const int nw = (int)g->schedule.size();
    int first = 0;
    for (size_t k = 0; k <= thresholds.size() && first < nw; ++k) {
        int end = nw;
        if (k < thresholds.size()) {
            end = first;
            while (end < nw && g->scheduleSize[end] > thresholds[k]) ++end;
        }
        if (end > first) plan.push_back(MakeClass(g, first, end - first, threads[k]));
        first = end;
    }
    return plan;
}

LaunchPlan DefaultPlan(const gb_world* g)
{
    const int nw = (int)g->schedule.size();
    // a single world: the widest CTA (its order-free phases scale with the width; configuration 2
    // coloured: 10.0 ms per step at 128 threads, 5.75 ms at 512)
    LaunchClass c{0, nw, nw == 1 ? 512 : 64, 640, 1024};
    return LaunchPlan{c};
}

std::vector<LaunchPlan> CandidatePlans(const gb_world* g)
{
    std::vector<LaunchPlan> c;
    c.push_back(DefaultPlan(g));
    if (g->schedule.size() < 2) {
        // one world: narrower CTAs too (the default is the widest)
        c.push_back(LaunchPlan{LaunchClass{0, 1, 256, 640, 1024}});
        c.push_back(LaunchPlan{LaunchClass{0, 1, 128, 640, 1024}});
        return c;
    }
    c.push_back(LaunchPlan{MakeClass(g, 0, (int)g->schedule.size(), 64)});
    c.push_back(SplitPlan(g, {160}, {64, 32}));
    c.push_back(SplitPlan(g, {256, 64}, {64, 64, 32}));
    c.push_back(SplitPlan(g, {320, 160, 64}, {128, 64, 32, 32}));
    // the largest worlds set the step's critical path: a small first class with wider CTAs
    c.push_back(SplitPlan(g, {400, 96}, {128, 64, 32}));
    c.push_back(SplitPlan(g, {320, 96}, {128, 64, 32}));
    c.push_back(SplitPlan(g, {400, 160}, {128, 64, 32}));
    c.push_back(SplitPlan(g, {400, 96}, {256, 64, 32}));
    c.push_back(SplitPlan(g, {320, 96}, {256, 64, 32}));
    c.push_back(SplitPlan(g, {400, 160, 64}, {256, 128, 64, 32}));
    c.push_back(SplitPlan(g, {320, 160, 64}, {256, 128, 64, 32}));
    // (classes with shared memory capped at 18-24 KB, for more resident worlds per SM, measured 15-25%
    // slower than the best plan on the bench batch: the solve's staging matters more)
    return c;
}

StepParams MakeParams(const gb_world* g, float dt, int vi, int pi)
{
    StepParams P;
    std::memset(&P, 0, sizeof(P));
    P.dt = dt;
    P.velocityIterations = vi;
    P.positionIterations = pi;
    P.maxToiEvents = g->maxToiEvents;
    P.solver = g->solver;
    P.tolerance = g->tolerance;
    P.measureResidual = g->measureResidual;
    P.warmMode = g->warmMode;
    P.mlp = g->mlp;
    P.logX = g->logX;
    P.logT = g->logT;
    P.logCount = g->logCount;
    P.logCap = g->logCap;
    P.recordEvents = g->eventsEnabled ? 1 : 0;
    return P;
}

void FreeLog(gb_world* g)
{
    if (g->logX) cudaFree(g->logX);
    if (g->logT) cudaFree(g->logT);
    if (g->logCount) cudaFree(g->logCount);
    g->logX = g->logT = nullptr;
    g->logCount = nullptr;
    g->logCap = 0;
}

gb_status EnsureSideStreams(gb_world* g, int n)
{
    if (!g->fork) GB_CUDA(cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming));
    for (int i = 1; i < n && i < kMaxClasses; ++i) {
        if (!g->side[i]) GB_CUDA(cudaStreamCreateWithFlags(&g->side[i], cudaStreamNonBlocking));
        if (!g->join[i]) GB_CUDA(cudaEventCreateWithFlags(&g->join[i], cudaEventDisableTiming));
    }
    return GB_OK;
}

// One per-world launch per class of the plan: class 0 (the largest worlds) on the handle's stream,
// submitted first so its CTAs are dispatched first, the others on side streams forked from the same
// point and joined back (a pattern stream capture records as one graph).
using ClassLaunch = cudaError_t (*)(const Batch&, const StepParams&, const int*, int, int, int, int, int, cudaStream_t);
gb_status LaunchClasses(gb_world* g, const StepParams& P, const LaunchPlan& plan, ClassLaunch launch)
{
    const int n = std::min((int)plan.size(), kMaxClasses);
    if (n > 1) {
        gb_status s = EnsureSideStreams(g, n);
        if (s != GB_OK) return s;
        GB_CUDA(cudaEventRecord(g->fork, g->stream));
    }
    if (n > 0) {
        const LaunchClass& c = plan[0];
        GB_CUDA(launch(g->batch, P, g->dSchedule, c.first, c.count, c.threads, c.rows, c.contacts, g->stream));
    }
    for (int i = 1; i < n; ++i) {
        const LaunchClass& c = plan[i];
        GB_CUDA(cudaStreamWaitEvent(g->side[i], g->fork, 0));
        GB_CUDA(launch(g->batch, P, g->dSchedule, c.first, c.count, c.threads, c.rows, c.contacts, g->side[i]));
        GB_CUDA(cudaEventRecord(g->join[i], g->side[i]));
    }
    for (int i = 1; i < n; ++i) GB_CUDA(cudaStreamWaitEvent(g->stream, g->join[i], 0));
    return GB_OK;
}

gb_status EnsurePipeStreams(gb_world* g, int n)
{
    if (!g->fork) GB_CUDA(cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming));
    int least = 0, greatest = 0;
    GB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    for (int i = 0; i < n && i < kMaxClasses; ++i) {
        // greatest is the numerically lowest value; class 0 (the largest worlds) gets it
        const int prio = std::min(greatest + i, least);
        if (!g->pipe[i]) GB_CUDA(cudaStreamCreateWithPriority(&g->pipe[i], cudaStreamNonBlocking, prio));
        if (!g->pipeJoin[i]) GB_CUDA(cudaEventCreateWithFlags(&g->pipeJoin[i], cudaEventDisableTiming));
    }
    return GB_OK;
}

// One step of every world with the given plan. Each class of the plan is a pipeline of its own on
// its own stream: the narrowphase pre-pass over its worlds' contact rows, the per-world step up to
// the continuous phase, the time-of-impact pre-pass over its worlds' rows, the per-world continuous
// phase. No stage waits for another class, so the continuous-phase tail of one class (a few worlds'
// event loops) overlaps the step of the others; stream priorities falling with the class keep the
// largest worlds' CTAs dispatched first. Worlds are independent, so any interleaving gives the
// same results.
gb_status LaunchPlanStep(gb_world* g, const StepParams& P, const LaunchPlan& plan)
{
    const int n = std::min((int)plan.size(), kMaxClasses);
    gb_status s = EnsurePipeStreams(g, n);
    if (s != GB_OK) return s;
    GB_CUDA(cudaEventRecord(g->fork, g->stream));
    for (int i = 0; i < n; ++i) {
        const LaunchClass& c = plan[i];
        cudaStream_t st = g->pipe[i];
        GB_CUDA(cudaStreamWaitEvent(st, g->fork, 0));
        // a split step (P.phase 1, then 2) runs the narrowphase and collide phase in its first half
        const int np0 = g->npChunkStart[c.first], toi0 = g->toiChunkStart[c.first];
        if (P.phase != 2)
            GB_CUDA(b2gLaunchNarrowphase(g->batch, g->dNpChunks + np0, g->npChunkStart[c.first + c.count] - np0, st));
        GB_CUDA(b2gLaunchStep(g->batch, P, g->dSchedule, c.first, c.count, c.threads, c.rows, c.contacts, st));
        if (P.phase != 1) {
            GB_CUDA(b2gLaunchToi(g->batch, P, g->dToiChunks + toi0, g->toiChunkStart[c.first + c.count] - toi0, st));
            GB_CUDA(b2gLaunchStepToi(g->batch, P, g->dSchedule, c.first, c.count, c.threads, c.rows, c.contacts, st));
        }
        GB_CUDA(cudaEventRecord(g->pipeJoin[i], st));
    }
    for (int i = 0; i < n; ++i) GB_CUDA(cudaStreamWaitEvent(g->stream, g->pipeJoin[i], 0));
    return GB_OK;
}

// A step of the online autotuner: the candidate under trial, timed with events on the handle's
// stream. Candidates take turns (rounds of one step each) so that the workload's drift over the
// tuning steps reaches all of them alike; after the last round the candidate with the smallest
// median time becomes the plan. tuneIndex is the candidate, tuneRep the round.
gb_status TunedStep(gb_world* g, const StepParams& P)
{
    const int nc = (int)g->candidates.size();
    const int trial = g->tuneIndex * g->tuneSteps + g->tuneRep;
    cudaEvent_t e0 = g->tuneEvents[2 * trial], e1 = g->tuneEvents[2 * trial + 1];
    GB_CUDA(cudaEventRecord(e0, g->stream));
    gb_status s = LaunchPlanStep(g, P, g->candidates[g->tuneIndex]);
    if (s != GB_OK) return s;
    GB_CUDA(cudaEventRecord(e1, g->stream));
    if (++g->tuneIndex == nc) { g->tuneIndex = 0; ++g->tuneRep; }
    if (g->tuneRep < g->tuneSteps) return GB_OK;
    g->tuneIndex = nc;
    GB_CUDA(cudaEventSynchronize(e1));
    int best = 0;
    for (int c = 0; c < nc; ++c) {
        std::vector<float> t(g->tuneSteps);
        for (int r = 0; r < g->tuneSteps; ++r) {
            const int k = c * g->tuneSteps + r;
            GB_CUDA(cudaEventElapsedTime(&t[r], g->tuneEvents[2 * k], g->tuneEvents[2 * k + 1]));
        }
        std::sort(t.begin(), t.end());
        g->candidateMs[c] = t[g->tuneSteps / 2];
        if (g->candidateMs[c] < g->candidateMs[best]) best = c;
    }
    g->plan = g->candidates[best];
    for (cudaEvent_t e : g->tuneEvents) cudaEventDestroy(e);
    g->tuneEvents.clear();
    g->tuneIndex = -1;
    return GB_OK;
}

void ReleaseGraph(gb_world* g)
{
    if (g->graph) cudaGraphExecDestroy(g->graph);
    g->graph = nullptr;
}

bool SamePlan(const LaunchPlan& a, const LaunchPlan& b)
{
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (a[i].first != b[i].first || a[i].count != b[i].count || a[i].threads != b[i].threads ||
            a[i].rows != b[i].rows || a[i].contacts != b[i].contacts)
            return false;
    return true;
}

// Streams, staging buffers and events of the pipelined transfers (after their work is done).
void ReleaseTransferResources(gb_world* g)
{
    if (g->upStream) { cudaStreamSynchronize(g->upStream); cudaStreamDestroy(g->upStream); }
    if (g->downStream) { cudaStreamSynchronize(g->downStream); cudaStreamDestroy(g->downStream); }
    g->upStream = g->downStream = nullptr;
    for (int i = 0; i < 2; ++i) {
        if (g->forceStage[i]) cudaFree(g->forceStage[i]);
        if (g->xfStage[i]) cudaFree(g->xfStage[i]);
        g->forceStage[i] = g->xfStage[i] = nullptr;
        for (cudaEvent_t* e : {&g->upDone[i], &g->forceTaken[i], &g->xfReady[i], &g->downDone[i]}) {
            if (*e) cudaEventDestroy(*e);
            *e = nullptr;
        }
    }
    g->stageBodies = 0;
}

void ReleaseLaunchResources(gb_world* g)
{
    ReleaseGraph(g);
    for (int i = 0; i < kMaxClasses; ++i) {
        if (g->side[i]) cudaStreamDestroy(g->side[i]);
        if (g->join[i]) cudaEventDestroy(g->join[i]);
        g->side[i] = nullptr;
        g->join[i] = nullptr;
    }
    for (int i = 0; i < kMaxClasses; ++i) {
        if (g->pipe[i]) cudaStreamDestroy(g->pipe[i]);
        if (g->pipeJoin[i]) cudaEventDestroy(g->pipeJoin[i]);
        g->pipe[i] = nullptr;
        g->pipeJoin[i] = nullptr;
    }
    if (g->fork) cudaEventDestroy(g->fork);
    g->fork = nullptr;
    for (cudaEvent_t e : g->tuneEvents) cudaEventDestroy(e);
    g->tuneEvents.clear();
    g->tuneIndex = -1;
}

// (Re)allocate device columns for the current world sizes and copy the host mirror over.
// The user contact filter's verdict table in the batch (or the default filter when none is set).
void AttachFilter(gb_world* g)
{
    Batch& B = g->batch;
    B.filterKeys = g->filterFn ? g->dFilterKeys : nullptr;
    B.filterVals = g->filterFn ? g->dFilterVals : nullptr;
    B.filterCap = g->filterFn ? g->filterCap : 0;
    B.filterMiss = g->filterFn ? g->dFilterMiss : nullptr;
    B.filterMissCap = 0;  // the host reads the pending verdicts from the table itself
}

void FreeFilter(gb_world* g)
{
    if (g->dFilterKeys) cudaFree(g->dFilterKeys);
    if (g->dFilterVals) cudaFree(g->dFilterVals);
    if (g->dFilterMiss) cudaFree(g->dFilterMiss);
    g->dFilterKeys = nullptr;
    g->dFilterVals = nullptr;
    g->dFilterMiss = nullptr;
    g->filterCap = g->filterUsed = 0;
}

// A verdict table of cap slots holding the given (key, value) entries.
gb_status BuildFilterTable(gb_world* g, int cap, const std::vector<unsigned long long>& keys, const std::vector<int>& vals)
{
    std::vector<unsigned long long> k((size_t)cap, ~0ull);
    std::vector<int> v((size_t)cap, 2);
    for (size_t i = 0; i < keys.size(); ++i) {
        unsigned slot = FilterSlot(keys[i], cap);
        while (k[slot] != ~0ull) slot = (slot + 1) & (unsigned)(cap - 1);
        k[slot] = keys[i];
        v[slot] = vals[i];
    }
    if (g->dFilterKeys) cudaFree(g->dFilterKeys);
    if (g->dFilterVals) cudaFree(g->dFilterVals);
    g->dFilterKeys = nullptr;
    g->dFilterVals = nullptr;
    GB_CUDA(cudaMalloc(&g->dFilterKeys, cap * sizeof(unsigned long long)));
    GB_CUDA(cudaMalloc(&g->dFilterVals, cap * sizeof(int)));
    GB_CUDA(cudaMemcpy(g->dFilterKeys, k.data(), cap * sizeof(unsigned long long), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(g->dFilterVals, v.data(), cap * sizeof(int), cudaMemcpyHostToDevice));
    g->filterCap = cap;
    g->filterUsed = (int)keys.size();
    return GB_OK;
}

// b2ContactFilter::ShouldCollide's default (Dynamics/b2WorldCallbacks.cpp:26-38) on the host mirror
bool HostDefaultFilter(const HWorld& W, int fA, int fB)
{
    const HFixture& a = W.fixtures[fA];
    const HFixture& b = W.fixtures[fB];
    if (a.group == b.group && a.group != 0) return a.group > 0;
    return (a.mask & b.category) != 0 && (a.category & b.mask) != 0;
}

gb_status Upload(gb_world* g)
{
    if (!g->hostDirty && g->onDevice) return GB_OK;
    if (!g->stream) {
        GB_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
        g->ownStream = true;
    }
    if (g->onDevice) { gb_status s = Download(g); if (s != GB_OK) return s; }
    FreeDevice(g);
    const int nw = (int)g->worlds.size();
    g->desc.assign(nw, WorldDesc{});
    long long tb = 0, tf = 0, tp = 0, tc = 0, tj = 0, tq = 0, tr = 0, tt = 0;
    for (int wi = 0; wi < nw; ++wi) {
        HWorld& W = g->worlds[wi];
        WorldDesc& d = g->desc[wi];
        d.bodyBase = (int)tb; d.bodyCount = (int)W.bodies.size();
        d.fixBase = (int)tf; d.fixCount = (int)W.fixtures.size();
        d.proxyBase = (int)tp; d.proxyCap = std::max(1, (int)W.fat.size());
        int oldCap = W.hasState ? (int)W.contacts.ci.size() : 0;
        int cap = std::max(64, 8 * d.fixCount);
        if (g->contactCapLimit > 0 && !W.hasState) cap = g->contactCapLimit;
        cap = std::max(std::max(cap, oldCap), W.capHint);
        d.contactBase = (int)tc; d.contactCap = cap;
        d.jointBase = (int)tj; d.jointCount = (int)W.joints.size();
        d.pairBase = (int)tq; d.pairCap = NextPow2(std::max(256, cap));
        d.rowBase = (int)tr; d.rowCap = d.bodyCount + cap + d.jointCount + 2 * kMaxTOIContacts;
        // island-DFS table: 29 bytes per body, a bit per contact slot, 16 bytes per table entry for up
        // to 8 entries per body (a world that needs more takes the DFS without a table)
        const long long islBytes = ((29ll * d.bodyCount + 4ll * ((cap + 31) / 32) + 16ll * (8ll * d.bodyCount + 64) +
                                     128) + 15) & ~15ll;
        d.islTabBase = tt; d.islTabBytes = (int)std::min<long long>(islBytes, 1ll << 30);
        tb += std::max(1, d.bodyCount); tf += std::max(1, d.fixCount); tp += d.proxyCap; tc += cap;
        tj += std::max(1, d.jointCount); tq += d.pairCap; tr += d.rowCap; tt += d.islTabBytes;
    }
    if (tb > (1LL << 31) - 1 || tc > (1LL << 31) - 1 || tq > (1LL << 31) - 1 || tr > (1LL << 31) - 1)
        return GB_ERR_CAPACITY;
    Batch& B = g->batch;
    B.worlds = nw;
    gb_status s = GB_OK;
#define ALLOC(field, n) if ((s = DevAlloc(g, &B.field, (size_t)(n))) != GB_OK) return s
    ALLOC(desc, nw); ALLOC(state, nw); ALLOC(bWorld, tb); ALLOC(cWorld, tc);
    B.bodyRows = (int)tb;
    B.contactRows = (int)tc;
    ALLOC(xf, tb); ALLOC(sw, tb); ALLOC(sw0, tb); ALLOC(vel, tb); ALLOC(frc, tb); ALLOC(mas, tb); ALLOC(prop, tb);
    ALLOC(bi, tb); ALLOC(bj, tb);
    ALLOC(fi, tf); ALLOC(fm, tf); ALLOC(ff, tf); ALLOC(faabb, tf); ALLOC(shape, tf);
    ALLOC(fat, tp); ALLOC(pfix, tp); ALLOC(moved, tp); ALLOC(movedList, tp); ALLOC(liveProxies, tp);
    ALLOC(gridIds, tp); ALLOC(gridNext, tp); ALLOC(gridPrev, tp); ALLOC(gridCellOf, tp); ALLOC(gridHead, tq + nw);
    ALLOC(ci, tc); ALLOC(ce, tc); ALLOC(cp, tc); ALLOC(mh, tc); ALLOC(mv, tc); ALLOC(mp0, tc); ALLOC(mp1, tc);
    ALLOC(order, 2 * tc); ALLOC(cnext, tc);
    ALLOC(joint, tj); ALLOC(sJoint, tj);
    ALLOC(sBody, tr); ALLOC(sStack, tb); ALLOC(sWake, tb); ALLOC(sPos, tr); ALLOC(sVel, tr); ALLOC(islands, tb);
    ALLOC(islandJ, tb); ALLOC(sleepOut, tb); ALLOC(rowMask, tr); ALLOC(sVelL, tr);
    ALLOC(sContact, tc); ALLOC(sStatus, tc); ALLOC(vc, tc); ALLOC(pc, tc); ALLOC(vimp, tc); ALLOC(vimpL, tc); ALLOC(vsep, tc); ALLOC(toi, tc); ALLOC(cColour, tc); ALLOC(colourList, tc);
    ALLOC(evType, tc);
    if (g->eventsEnabled) { ALLOC(evLog, 8 * tc); } else { B.evLog = nullptr; }
    if (g->treeTrack) {
        ALLOC(treeLogId, kTreeLogPerProxy * tp + (long long)kTreeLogExtra * nw);
        ALLOC(treeLogFat, kTreeLogPerProxy * tp + (long long)kTreeLogExtra * nw);
    } else {
        B.treeLogId = nullptr;
        B.treeLogFat = nullptr;
    }
    ALLOC(pairs, tq); ALLOC(pairKeep, tq); ALLOC(pairInfo, tq); ALLOC(islTab, tt);
#undef ALLOC
    GB_CUDA(cudaMemcpy(B.desc, g->desc.data(), nw * sizeof(WorldDesc), cudaMemcpyHostToDevice));
    std::vector<WorldState> states(nw);
    // Host staging of every column for all worlds, then one copy per column.
    std::vector<float4> xf(tb), sw(tb), sw0(tb), vel(tb), frc(tb), mas(tb), prop(tb);
    std::vector<int4> bi(tb, make_int4(0, 0, kNullIdx, kNullIdx)), bj(tb, make_int4(kNullIdx, kNullIdx, 0, 0));
    std::vector<int4> fi(tf, make_int4(kNullIdx, kNullIdx, kNullIdx, 0)), ff(tf);
    std::vector<float4> fm(tf), faabb(tf);
    std::vector<Shape> shapes(tf);
    std::vector<float4> fat(tp, make_float4(0, 0, 0, 0));
    std::vector<int> pfix(tp, kNullIdx), moved(tp, 0);
    std::vector<int4> ci(tc, make_int4(0, 0, 0, 0)), ce(tc, make_int4(-1, -1, -1, -1)), mh(tc, make_int4(0, 0, 0, 0));
    std::vector<float4> cp(tc, make_float4(0, 0, 0, 1)), mv(tc), mp0(tc), mp1(tc);
    std::vector<int> order(2 * tc, 0), cnext(tc, kNullIdx);
    std::vector<Joint> joints(tj);
    for (int wi = 0; wi < nw; ++wi) {
        HWorld& W = g->worlds[wi];
        const WorldDesc& d = g->desc[wi];
        for (int i = 0; i < d.bodyCount; ++i) {
            const HBody& b = W.bodies[i];
            const int r = d.bodyBase + i;
            xf[r] = make_float4(b.xf.p.x, b.xf.p.y, b.xf.q.s, b.xf.q.c);
            sw[r] = make_float4(b.sw.c.x, b.sw.c.y, b.sw.a, b.sw.alpha0);
            sw0[r] = make_float4(b.sw.c0.x, b.sw.c0.y, b.sw.a0, b.sleepTime);
            vel[r] = make_float4(b.v.x, b.v.y, b.w, 0.0f);
            frc[r] = make_float4(b.force.x, b.force.y, b.torque, 0.0f);
            mas[r] = make_float4(b.invMass, b.invI, b.sw.localCenter.x, b.sw.localCenter.y);
            prop[r] = make_float4(b.linDamp, b.angDamp, b.gravScale, b.mass);
            bi[r] = make_int4(b.type, b.flags, b.fixtureList, W.hasState ? b.contactList : kNullIdx);
            bj[r] = make_int4(b.jointList, b.next, 0, 0);
        }
        for (int i = 0; i < d.fixCount; ++i) {
            const HFixture& f = W.fixtures[i];
            const int r = d.fixBase + i;
            fi[r] = make_int4(f.body, f.next, f.proxyId, f.sensor);
            fm[r] = make_float4(f.friction, f.restitution, f.density, f.shape.radius);
            ff[r] = make_int4(f.category, f.mask, f.group, 0);
            faabb[r] = f.aabb;
            shapes[r] = f.shape;
        }
        const int np = d.proxyCap;
        W.fat.resize(np, make_float4(0, 0, 0, 0)); W.pfix.resize(np, kNullIdx); W.moved.resize(np, 0);
        std::copy(W.fat.begin(), W.fat.end(), fat.begin() + d.proxyBase);
        std::copy(W.pfix.begin(), W.pfix.end(), pfix.begin() + d.proxyBase);
        std::copy(W.moved.begin(), W.moved.end(), moved.begin() + d.proxyBase);
        // contacts: previous slots keep their index; the rest of the capacity joins the free list
        const int cap = d.contactCap;
        HContacts& C = W.contacts;
        const int old = W.hasState ? (int)C.ci.size() : 0;
        for (int i = 0; i < old; ++i) {
            const int r = d.contactBase + i;
            ci[r] = C.ci[i]; ce[r] = C.ce[i]; mh[r] = C.mh[i]; cp[r] = C.cp[i]; mv[r] = C.mv[i];
            mp0[r] = C.mp0[i]; mp1[r] = C.mp1[i]; cnext[r] = C.cnext[i];
        }
        WorldState st = W.hasState ? W.state : WorldState{};
        {
            // the contact list at the end of the world's 2 x cap order rows (room to prepend in front)
            const int live = W.hasState ? st.contactCount : 0;
            st.orderStart = 2 * cap - live;
            for (int i = 0; i < live; ++i) order[2 * (size_t)d.contactBase + st.orderStart + i] = C.order[i];
        }
        int freeHead = W.hasState ? W.state.freeContact : kNullIdx;
        for (int i = cap - 1; i >= old; --i) { cnext[d.contactBase + i] = freeHead; freeHead = i; }
        if (!W.hasState) st.contactCount = 0;
        st.freeContact = freeHead;
        st.gx = W.def.gravity_x; st.gy = W.def.gravity_y;
        st.bodyList = W.bodyList;
        st.jointList = W.jointList;
        st.newFixture = W.newFixture;
        if (!W.hasState) { st.stepComplete = 1; st.inv_dt0 = 0.0f; }
        st.allowSleep = W.def.allow_sleep; st.warmStarting = W.def.warm_starting;
        st.continuous = W.def.continuous_physics; st.subStepping = W.def.sub_stepping;
        st.clearForces = W.autoClear ? 1 : 0;
        st.error = 0;
        st.gridValid = 0;
        st.treeLogCount = 0;
        states[wi] = st;
        for (int j = 0; j < d.jointCount; ++j) joints[d.jointBase + j] = W.joints[j];
        W.hasState = true;
        W.state = st;
        C = HContacts();
    }
    if ((s = Put(B.xf, xf, tb)) != GB_OK || (s = Put(B.sw, sw, tb)) != GB_OK || (s = Put(B.sw0, sw0, tb)) != GB_OK ||
        (s = Put(B.vel, vel, tb)) != GB_OK || (s = Put(B.frc, frc, tb)) != GB_OK || (s = Put(B.mas, mas, tb)) != GB_OK ||
        (s = Put(B.prop, prop, tb)) != GB_OK || (s = Put(B.bi, bi, tb)) != GB_OK || (s = Put(B.bj, bj, tb)) != GB_OK ||
        (s = Put(B.fi, fi, tf)) != GB_OK || (s = Put(B.fm, fm, tf)) != GB_OK || (s = Put(B.ff, ff, tf)) != GB_OK ||
        (s = Put(B.faabb, faabb, tf)) != GB_OK || (s = Put(B.shape, shapes, tf)) != GB_OK ||
        (s = Put(B.fat, fat, tp)) != GB_OK || (s = Put(B.pfix, pfix, tp)) != GB_OK || (s = Put(B.moved, moved, tp)) != GB_OK ||
        (s = Put(B.ci, ci, tc)) != GB_OK || (s = Put(B.ce, ce, tc)) != GB_OK || (s = Put(B.mh, mh, tc)) != GB_OK ||
        (s = Put(B.cp, cp, tc)) != GB_OK || (s = Put(B.mv, mv, tc)) != GB_OK || (s = Put(B.mp0, mp0, tc)) != GB_OK ||
        (s = Put(B.mp1, mp1, tc)) != GB_OK || (s = Put(B.order, order, 2 * tc)) != GB_OK ||
        (s = Put(B.cnext, cnext, tc)) != GB_OK || (s = Put(B.joint, joints, tj)) != GB_OK)
        return s;
    GB_CUDA(cudaMemcpy(B.state, states.data(), nw * sizeof(WorldState), cudaMemcpyHostToDevice));
    {
        // row -> world maps of the body and contact columns (padding rows belong to their world)
        std::vector<int> bw(tb), cw(tc);
        for (int wi = 0; wi < nw; ++wi) {
            const WorldDesc& d = g->desc[wi];
            std::fill(bw.begin() + d.bodyBase, bw.begin() + d.bodyBase + std::max(1, d.bodyCount), wi);
            std::fill(cw.begin() + d.contactBase, cw.begin() + d.contactBase + d.contactCap, wi);
        }
        if ((s = Put(B.bWorld, bw, tb)) != GB_OK || (s = Put(B.cWorld, cw, tc)) != GB_OK) return s;
    }
    // Largest worlds first: with one CTA per world the longest step starts earliest.
    std::vector<int> schedule(nw);
    std::iota(schedule.begin(), schedule.end(), 0);
    std::stable_sort(schedule.begin(), schedule.end(), [&](int a, int b) {
        return g->desc[a].fixCount > g->desc[b].fixCount;
    });
    if ((s = DevAlloc(g, &g->dSchedule, nw)) != GB_OK) return s;
    GB_CUDA(cudaMemcpy(g->dSchedule, schedule.data(), nw * sizeof(int), cudaMemcpyHostToDevice));
    {
        // row chunks of the flat pre-passes, world by world in schedule order: the narrowphase's over
        // contact rows, the time-of-impact pass's over body rows (at least one) then contact rows
        std::vector<int4> np, toi;
        g->npChunkStart.assign(nw + 1, 0);
        g->toiChunkStart.assign(nw + 1, 0);
        for (int slot = 0; slot < nw; ++slot) {
            const int w = schedule[slot];
            const WorldDesc& d = g->desc[w];
            g->npChunkStart[slot] = (int)np.size();
            g->toiChunkStart[slot] = (int)toi.size();
            const int bodyRows = std::max(1, d.bodyCount);
            for (int k = 0; k < d.contactCap; k += kRowChunk)
                np.push_back(make_int4(w, k, std::min(kRowChunk, d.contactCap - k), 0));
            for (int k = 0; k < bodyRows; k += kRowChunk)
                toi.push_back(make_int4(w, k, std::min(kRowChunk, bodyRows - k), 0));
            for (int k = 0; k < d.contactCap; k += kRowChunk)
                toi.push_back(make_int4(w, k, std::min(kRowChunk, d.contactCap - k), 1));
        }
        g->npChunkStart[nw] = (int)np.size();
        g->toiChunkStart[nw] = (int)toi.size();
        if ((s = DevAlloc(g, &g->dNpChunks, np.size())) != GB_OK) return s;
        if ((s = DevAlloc(g, &g->dToiChunks, toi.size())) != GB_OK) return s;
        if (!np.empty())
            GB_CUDA(cudaMemcpy(g->dNpChunks, np.data(), np.size() * sizeof(int4), cudaMemcpyHostToDevice));
        if (!toi.empty())
            GB_CUDA(cudaMemcpy(g->dToiChunks, toi.data(), toi.size() * sizeof(int4), cudaMemcpyHostToDevice));
    }
    g->schedule = schedule;
    g->scheduleSize.resize(nw);
    for (int i = 0; i < nw; ++i) g->scheduleSize[i] = g->desc[schedule[i]].bodyCount;
    g->plan = DefaultPlan(g);
    g->onDevice = true;
    g->hostDirty = false;
    AttachFilter(g);
    return GB_OK;
}

// A step with a user contact filter. The device takes the default filter's verdict for pairs the
// table does not know yet and logs that it met them; afterwards the user's filter decides each such
// pair (b2ContactFilter::ShouldCollide, called here on the host with the ordered fixture pair). When
// every decision equals the default's the step stands; otherwise every device column is restored
// from the copy taken before the step and the step runs again with the decisions known (a bounded
// number of times: each run leaves more pairs decided). The filter must give the same verdict for
// the same ordered fixture pair until gb_world_refilter says otherwise.
gb_status FilteredStep(gb_world* g, const StepParams& P)
{
    if (g->shadow.size() != g->allocations.size()) {
        for (void* p : g->shadow) cudaFree(p);
        g->shadow.assign(g->allocations.size(), nullptr);
        for (size_t i = 0; i < g->allocations.size(); ++i)
            GB_CUDA(cudaMalloc(&g->shadow[i], g->allocationBytes[i]));
    }
    for (int attempt = 0; attempt < 16; ++attempt) {
        for (size_t i = 0; i < g->allocations.size(); ++i)
            GB_CUDA(cudaMemcpyAsync(g->shadow[i], g->allocations[i], g->allocationBytes[i], cudaMemcpyDeviceToDevice,
                                    g->stream));
        GB_CUDA(cudaMemsetAsync(g->dFilterMiss, 0, sizeof(int), g->stream));
        gb_status s = LaunchPlanStep(g, P, g->plan);
        if (s != GB_OK) return s;
        int missed = 0;
        GB_CUDA(cudaMemcpyAsync(&missed, g->dFilterMiss, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
        GB_CUDA(cudaStreamSynchronize(g->stream));
        if (missed == 0) return GB_OK;
        // every pending verdict of the table, decided by the user's filter
        std::vector<unsigned long long> keys((size_t)g->filterCap);
        std::vector<int> vals((size_t)g->filterCap);
        GB_CUDA(cudaMemcpy(keys.data(), g->dFilterKeys, g->filterCap * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(vals.data(), g->dFilterVals, g->filterCap * sizeof(int), cudaMemcpyDeviceToHost));
        bool differs = false;
        std::vector<unsigned long long> allKeys;
        std::vector<int> allVals;
        for (int i = 0; i < g->filterCap; ++i) {
            if (keys[i] == ~0ull) continue;
            if (vals[i] == 2) {
                const int w = (int)(keys[i] >> 40), fA = (int)((keys[i] >> 20) & 0xFFFFF), fB = (int)(keys[i] & 0xFFFFF);
                vals[i] = g->filterFn(g->filterUser, w, fA, fB) ? 1 : 0;
                if ((vals[i] != 0) != HostDefaultFilter(g->worlds[w], fA, fB)) differs = true;
            }
            allKeys.push_back(keys[i]);
            allVals.push_back(vals[i]);
        }
        int cap = g->filterCap;
        while ((int)allKeys.size() * 2 > cap) cap *= 2;  // keep the table at most half full
        s = BuildFilterTable(g, cap, allKeys, allVals);
        if (s != GB_OK) return s;
        AttachFilter(g);
        if (!differs) return GB_OK;
        ++g->filterReplays;
        ReleaseGraph(g);
        for (size_t i = 0; i < g->allocations.size(); ++i)
            GB_CUDA(cudaMemcpyAsync(g->allocations[i], g->shadow[i], g->allocationBytes[i], cudaMemcpyDeviceToDevice,
                                    g->stream));
    }
    return GB_ERR_TIMEOUT;
}

// One step with grow-and-retry: every device column is copied aside, the step runs and is waited for,
// and when a world overflowed a fixed buffer (GB_ERR_CAPACITY: contact slots, pairs, island rows) or
// hit the time-of-impact event limit (GB_ERR_TIMEOUT), the columns are put back, the world's contact
// capacity (which sizes the pair and row buffers too) or the event limit is doubled, the state goes
// through the host to the larger buffers, and the step runs again; the overflowing attempt leaves no
// trace, so the result is the step the reference takes. After recoverAttempts retries the last
// error stands, as without recovery.
gb_status StepOnce(gb_world* g, const StepParams& P)
{
    if (g->filterFn) return FilteredStep(g, P);
    if (g->tuneIndex >= 0) return TunedStep(g, P);
    return LaunchPlanStep(g, P, g->plan);
}

gb_status RecoveringStep(gb_world* g, float dt, int vi, int pi)
{
    for (int attempt = 0;; ++attempt) {
        if (g->recoverShadow.size() != g->allocations.size()) {
            for (void* p : g->recoverShadow) cudaFree(p);
            g->recoverShadow.assign(g->allocations.size(), nullptr);
            for (size_t i = 0; i < g->allocations.size(); ++i)
                GB_CUDA(cudaMalloc(&g->recoverShadow[i], g->allocationBytes[i]));
        }
        for (size_t i = 0; i < g->allocations.size(); ++i)
            GB_CUDA(cudaMemcpyAsync(g->recoverShadow[i], g->allocations[i], g->allocationBytes[i],
                                    cudaMemcpyDeviceToDevice, g->stream));
        gb_status s = StepOnce(g, MakeParams(g, dt, vi, pi));
        if (s != GB_OK) return s;
        GB_CUDA(cudaStreamSynchronize(g->stream));
        const int nw = (int)g->worlds.size();
        std::vector<WorldState> st(nw);
        GB_CUDA(cudaMemcpy(st.data(), g->batch.state, nw * sizeof(WorldState), cudaMemcpyDeviceToHost));
        bool capacity = false, timeout = false;
        for (const WorldState& x : st) {
            capacity |= (x.error & kErrCapacity) != 0;
            timeout |= (x.error & kErrTimeout) != 0;
        }
        if (!capacity && !timeout) return GB_OK;
        if (attempt >= g->recoverAttempts) return GB_OK;  // the error stays in the state for gb_world_sync
        for (size_t i = 0; i < g->allocations.size(); ++i)
            GB_CUDA(cudaMemcpyAsync(g->allocations[i], g->recoverShadow[i], g->allocationBytes[i],
                                    cudaMemcpyDeviceToDevice, g->stream));
        GB_CUDA(cudaStreamSynchronize(g->stream));
        for (int wi = 0; wi < nw; ++wi)
            if (st[wi].error & kErrCapacity)
                g->worlds[wi].capHint = 2 * g->desc[wi].contactCap;
        if (timeout) {
            g->maxToiEvents *= 2;
            ReleaseGraph(g);
        }
        ++g->recoveries;
        s = Download(g);
        if (s != GB_OK) return s;
        g->hostDirty = true;
        s = Upload(g);
        if (s != GB_OK) return s;
    }
}

gb_status Mutable(gb_world* g, int w)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || g->locked) return GB_ERR_INVALID;
    if (g->onDevice) {
        gb_status s = Download(g);
        if (s != GB_OK) return s;
    }
    g->hostDirty = true;
    return GB_OK;
}

gb_status CreateBody(HWorld& W, int type, const float* f, int fl, int* id)
{
    if (type < 0 || type > 2) return GB_ERR_INVALID;
    HBody b;
    b.type = type;
    b.flags = 0;
    if (fl & 8) b.flags |= kBBullet;
    if (fl & 4) b.flags |= kBFixedRot;
    if (fl & 1) b.flags |= kBAutoSleep;
    if (fl & 2) b.flags |= kBAwake;
    if (fl & 16) b.flags |= kBActive;
    // b2Body::b2Body (Box2D/Dynamics/b2Body.cpp:27-107)
    b.xf.p = V(f[0], f[1]);
    b.xf.q = RotOf(f[2]);
    b.sw.localCenter = V(0.0f, 0.0f);
    b.sw.c0 = b.xf.p; b.sw.c = b.xf.p;
    b.sw.a0 = f[2]; b.sw.a = f[2]; b.sw.alpha0 = 0.0f;
    b.v = V(f[3], f[4]); b.w = f[5];
    b.linDamp = f[6]; b.angDamp = f[7]; b.gravScale = f[8];
    if (type == kDynamic) { b.mass = 1.0f; b.invMass = 1.0f; }
    int idx = (int)W.bodies.size();
    b.next = W.bodyList;
    W.bodyList = idx;
    W.bodies.push_back(b);
    if (id) *id = idx;
    return GB_OK;
}

gb_status CreateFixture(HWorld& W, int body, int type, const float* s, int n, const float* mat, const int* filt, int* id)
{
    if (body < 0 || body >= (int)W.bodies.size() || type < 0 || type > 3) return GB_ERR_INVALID;
    if ((type == 2 && (n < 3 || n > kMaxPolyVerts))) return GB_ERR_INVALID;
    HFixture fx;
    fx.body = body;
    fx.shape = MakeShape(type, s, n);
    // a chain's next child follows the previous child of the same body
    const int prevChild = (int)W.fixtures.size() - 1;
    if (type == 1 && !(s[10] == 0.0f || s[10] == 1.0f || s[10] == 2.0f)) return GB_ERR_INVALID;
    if (type == 1 && fx.shape.chain == 2 &&
        (prevChild < 0 || W.fixtures[prevChild].body != body || W.fixtures[prevChild].shape.type != kEdge ||
         W.fixtures[prevChild].shape.chain == 0))
        return GB_ERR_INVALID;
    fx.density = mat[0]; fx.friction = mat[1]; fx.restitution = mat[2];
    fx.category = filt[0] & 0xFFFF; fx.mask = filt[1] & 0xFFFF; fx.group = (int16_t)filt[2]; fx.sensor = filt[3] != 0;
    int idx = (int)W.fixtures.size();
    HBody& b = W.bodies[body];
    if (b.flags & kBActive) {
        // b2Fixture::CreateProxies (Box2D/Dynamics/b2Fixture.cpp:121-137) + b2DynamicTree::CreateProxy
        fx.aabb = ComputeAABB(fx.shape, b.xf);
        float4 fat = make_float4(fx.aabb.x - kAabbExtension, fx.aabb.y - kAabbExtension,
                                 fx.aabb.z + kAabbExtension, fx.aabb.w + kAabbExtension);
        fx.proxyId = AllocateProxy(W, fat, idx);
    }
    if (fx.shape.type == kEdge && fx.shape.chain == 2) {
        // after the previous child: the body's list visits a chain's children in ascending order, as
        // b2Fixture::Synchronize moves them (b2Fixture.cpp:154-177)
        fx.next = W.fixtures[prevChild].next;
        W.fixtures[prevChild].next = idx;
    } else {
        fx.next = b.fixtureList;
        b.fixtureList = idx;
    }
    W.fixtures.push_back(fx);
    if (fx.density > 0.0f) ResetMassData(W, body);
    W.newFixture = 1;
    if (id) *id = idx;
    return GB_OK;
}

// b2World::CreateJoint (Dynamics/b2World.cpp:185-250) for any joint definition; f as gb_create_joints
// documents.
gb_status CreateJoint(HWorld& W, int type, int a, int b, const float* f, int fl, int* id)
{
    int nb = (int)W.bodies.size();
    if (a < 0 || a >= nb || b < 0 || b >= nb || a == b) return GB_ERR_INVALID;
    if (type < 0 || type >= kJointTypes) return GB_ERR_INVALID;
    Joint j;
    std::memset(&j, 0, sizeof(j));
    j.type = type;
    j.bodyA = a; j.bodyB = b;
    j.localAnchorA = V(f[0], f[1]); j.localAnchorB = V(f[2], f[3]);
    if (type == kJointRevolute) {
        j.referenceAngle = f[4]; j.lowerAngle = f[5]; j.upperAngle = f[6]; j.motorSpeed = f[7]; j.maxMotorTorque = f[8];
        j.enableLimit = (fl & 1) != 0; j.enableMotor = (fl & 2) != 0;
    } else if (type == kJointDistance) {
        j.length = f[4]; j.frequencyHz = f[5]; j.dampingRatio = f[6];
    } else if (type == kJointWeld) {
        j.referenceAngle = f[4]; j.frequencyHz = f[5]; j.dampingRatio = f[6];
    } else if (type == kJointWheel) {
        // b2WheelJoint::b2WheelJoint (Dynamics/Joints/b2WheelJoint.cpp:39-64): the axis as given, its
        // normal b2Cross(1, axis)
        j.localXAxisA = V(f[4], f[5]);
        j.localYAxisA = Cross(1.0f, j.localXAxisA);
        j.maxMotorTorque = f[6]; j.motorSpeed = f[7]; j.frequencyHz = f[8]; j.dampingRatio = f[9];
        j.enableMotor = (fl & 2) != 0;
    } else if (type == kJointMouse) {
        // b2MouseJoint::b2MouseJoint (Dynamics/Joints/b2MouseJoint.cpp:33-52): the target's point on
        // body B at creation
        j.target = V(f[0], f[1]);
        j.localAnchorA = V(0.0f, 0.0f);
        j.localAnchorB = MulT(W.bodies[b].xf, j.target);
        j.maxForce = f[2]; j.frequencyHz = f[3]; j.dampingRatio = f[4];
    } else if (type == kJointPulley) {
        // b2PulleyJoint::b2PulleyJoint (b2PulleyJoint.cpp:53-69)
        j.groundAnchorA = V(f[0], f[1]); j.groundAnchorB = V(f[2], f[3]);
        j.localAnchorA = V(f[4], f[5]); j.localAnchorB = V(f[6], f[7]);
        j.lengthA = f[8]; j.lengthB = f[9]; j.ratio = f[10];
        if (!(j.ratio != 0.0f)) return GB_ERR_INVALID;
        j.pulleyConstant = f[8] + j.ratio * f[9];
    } else if (type == kJointGear) {
        // b2GearJoint::b2GearJoint (Dynamics/Joints/b2GearJoint.cpp:49-136): f[0], f[1] the indices of
        // two existing revolute or prismatic joints, f[2] the ratio. Bodies A and B become the joints'
        // bodies B (the joint edges go there), C and D their bodies A; the constant is the coordinates'
        // combination at creation.
        const int j1 = (int)f[0], j2 = (int)f[1];
        const int nj = (int)W.joints.size();
        if ((float)j1 != f[0] || (float)j2 != f[1] || j1 < 0 || j1 >= nj || j2 < 0 || j2 >= nj) return GB_ERR_INVALID;
        const Joint& J1 = W.joints[j1];
        const Joint& J2 = W.joints[j2];
        if ((J1.type != kJointRevolute && J1.type != kJointPrismatic) ||
            (J2.type != kJointRevolute && J2.type != kJointPrismatic))
            return GB_ERR_INVALID;
        j.gearTypeA = J1.type; j.gearTypeB = J2.type;
        j.bodyC = J1.bodyA; j.bodyA = J1.bodyB;
        j.bodyD = J2.bodyA; j.bodyB = J2.bodyB;
        const HBody &bA = W.bodies[j.bodyA], &bC = W.bodies[j.bodyC];
        const HBody &bB = W.bodies[j.bodyB], &bD = W.bodies[j.bodyD];
        j.localAnchorC = J1.localAnchorA; j.localAnchorA = J1.localAnchorB; j.referenceAngle = J1.referenceAngle;
        j.localAnchorD = J2.localAnchorA; j.localAnchorB = J2.localAnchorB; j.referenceAngleB = J2.referenceAngle;
        float coordinateA, coordinateB;
        if (J1.type == kJointRevolute) {
            j.localAxisC = V(0.0f, 0.0f);
            coordinateA = bA.sw.a - bC.sw.a - j.referenceAngle;
        } else {
            j.localAxisC = J1.localXAxisA;
            const Vec2 pA = MulT(bC.xf.q, Mul(bA.xf.q, j.localAnchorA) + (bA.xf.p - bC.xf.p));
            coordinateA = Dot(pA - j.localAnchorC, j.localAxisC);
        }
        if (J2.type == kJointRevolute) {
            j.localAxisD = V(0.0f, 0.0f);
            coordinateB = bB.sw.a - bD.sw.a - j.referenceAngleB;
        } else {
            j.localAxisD = J2.localXAxisA;
            const Vec2 pB = MulT(bD.xf.q, Mul(bB.xf.q, j.localAnchorB) + (bB.xf.p - bD.xf.p));
            coordinateB = Dot(pB - j.localAnchorD, j.localAxisD);
        }
        j.ratio = f[2];
        j.gearConstant = coordinateA + j.ratio * coordinateB;
    } else if (type == kJointRope) {
        j.maxLength = f[4];  // b2RopeJoint::b2RopeJoint (b2RopeJoint.cpp:35-45)
    } else if (type == kJointFriction) {
        j.maxForce = f[4]; j.maxTorque = f[5];  // b2FrictionJoint::b2FrictionJoint (b2FrictionJoint.cpp:35-45)
    } else if (type == kJointMotor) {
        // b2MotorJoint::b2MotorJoint (b2MotorJoint.cpp:43-56): no anchors; the offsets in f[0..2]
        j.localAnchorA = V(0.0f, 0.0f); j.localAnchorB = V(0.0f, 0.0f);
        j.linearOffset = V(f[0], f[1]); j.angularOffset = f[2];
        j.maxForce = f[3]; j.maxTorque = f[4]; j.correctionFactor = f[5];
    } else {
        // b2PrismaticJoint::b2PrismaticJoint (Dynamics/Joints/b2PrismaticJoint.cpp:102-126): the unit
        // axis (b2Vec2::Normalize), its normal b2Cross(1, axis); the translation limits and the motor
        // force sit in the angle-limit and motor-torque fields
        Vec2 axis = V(f[4], f[5]);
        Normalize(axis);
        j.localXAxisA = axis;
        j.localYAxisA = Cross(1.0f, axis);
        j.referenceAngle = f[6]; j.lowerAngle = f[7]; j.upperAngle = f[8];
        j.maxMotorTorque = f[9]; j.motorSpeed = f[10];
        j.enableLimit = (fl & 1) != 0; j.enableMotor = (fl & 2) != 0;
    }
    j.collideConnected = (fl & 4) != 0;
    int idx = (int)W.joints.size();
    j.prev = kNullIdx;
    j.next = W.jointList;
    if (W.jointList != kNullIdx) W.joints[W.jointList].prev = idx;
    W.jointList = idx;
    // edge 2*idx on bodyA's joint list, 2*idx+1 on bodyB's (b2World.cpp:212-236); the joint's bodies,
    // which for a gear joint are not the definition's
    for (int side = 0; side < 2; ++side) {
        HBody& body = W.bodies[side == 0 ? j.bodyA : j.bodyB];
        int e = 2 * idx + side;
        j.ePrev[side] = kNullIdx;
        j.eNext[side] = body.jointList;
        if (body.jointList != kNullIdx) W.joints[body.jointList >> 1].ePrev[body.jointList & 1] = e;
        body.jointList = e;
    }
    W.joints.push_back(j);
    // Contacts between the definition's two bodies are flagged for filtering (b2World.cpp:238-250).
    if (!j.collideConnected && W.hasState) {
        HContacts& C = W.contacts;
        for (int e = W.bodies[b].contactList; e != kNullIdx;) {
            int c = e >> 1;
            int4 info = C.ci[c];
            int other = (e & 1) == 0 ? W.fixtures[info.z].body : W.fixtures[info.y].body;
            if (other == a) C.ci[c].x |= kCFilter;
            int4 v = C.ce[c];
            e = (e & 1) ? v.w : v.y;
        }
    }
    if (id) *id = idx;
    return GB_OK;
}

// ------------------------------------------------------------------ destruction (host mirror)
// The listener calls a destruction makes, in order: {0, joint, 0} SayGoodbye(joint), {1, fixture, 0}
// SayGoodbye(fixture), {2, fixtureA, fixtureB} EndContact.
using Calls = std::vector<int>;

void WakeHost(HBody& b)
{
    if ((b.flags & kBAwake) == 0) {
        b.flags |= kBAwake;
        b.sleepTime = 0.0f;
    }
}

// b2ContactManager::Destroy + b2Contact::Destroy (Dynamics/b2ContactManager.cpp:46-104,
// Contacts/b2Contact.cpp:102-125) on the pulled-back contact columns: EndContact when touching, out
// of the world list (order kept) and both bodies' edge lists, both bodies woken when the manifold had
// points and neither fixture is a sensor, the slot back to the free list.
void DestroyContactHost(HWorld& W, int c, Calls& calls)
{
    HContacts& C = W.contacts;
    const int4 info = C.ci[c];
    const int fA = info.y, fB = info.z;
    const int bA = W.fixtures[fA].body, bB = W.fixtures[fB].body;
    if (info.x & kCTouching) calls.insert(calls.end(), {2, fA, fB});
    const int n = W.state.contactCount;
    int k = 0;
    while (k < n && C.order[k] != c) ++k;
    for (; k + 1 < n; ++k) C.order[k] = C.order[k + 1];
    W.state.contactCount = n - 1;
    for (int side = 0; side < 2; ++side) {
        HBody& body = W.bodies[side == 0 ? bA : bB];
        const int e = 2 * c + side;
        const int4 v = C.ce[c];
        const int pe = side == 0 ? v.x : v.z, ne = side == 0 ? v.y : v.w;
        if (pe != kNullIdx) (pe & 1 ? C.ce[pe >> 1].w : C.ce[pe >> 1].y) = ne;
        if (ne != kNullIdx) (ne & 1 ? C.ce[ne >> 1].z : C.ce[ne >> 1].x) = pe;
        if (body.contactList == e) body.contactList = ne;
    }
    if (C.mh[c].y > 0 && !W.fixtures[fA].sensor && !W.fixtures[fB].sensor) {
        WakeHost(W.bodies[bA]);
        WakeHost(W.bodies[bB]);
    }
    C.ci[c] = make_int4(0, 0, 0, 0);
    C.ce[c] = make_int4(kNullIdx, kNullIdx, kNullIdx, kNullIdx);
    C.cnext[c] = W.state.freeContact;
    W.state.freeContact = c;
}

// b2World::DestroyJoint (Dynamics/b2World.cpp:274-362). The slot stays, with no bodies.
void DestroyJointHost(HWorld& W, int jn)
{
    Joint& j = W.joints[jn];
    const bool collideConnected = j.collideConnected;
    if (j.prev != kNullIdx) W.joints[j.prev].next = j.next;
    if (j.next != kNullIdx) W.joints[j.next].prev = j.prev;
    if (W.jointList == jn) W.jointList = j.next;
    const int bA = j.bodyA, bB = j.bodyB;
    WakeHost(W.bodies[bA]);
    WakeHost(W.bodies[bB]);
    for (int side = 0; side < 2; ++side) {
        HBody& body = W.bodies[side == 0 ? bA : bB];
        const int e = 2 * jn + side;
        const int pe = j.ePrev[side], ne = j.eNext[side];
        if (pe != kNullIdx) W.joints[pe >> 1].eNext[pe & 1] = ne;
        if (ne != kNullIdx) W.joints[ne >> 1].ePrev[ne & 1] = pe;
        if (body.jointList == e) body.jointList = ne;
        j.ePrev[side] = j.eNext[side] = kNullIdx;
    }
    j.prev = j.next = kNullIdx;
    j.bodyA = j.bodyB = kNullIdx;
    j.islandFlag = 0;
    if (!collideConnected && W.hasState) {
        HContacts& C = W.contacts;
        for (int e = W.bodies[bB].contactList; e != kNullIdx;) {
            const int c = e >> 1;
            const int4 info = C.ci[c];
            const int other = (e & 1) == 0 ? W.fixtures[info.z].body : W.fixtures[info.y].body;
            if (other == bA) C.ci[c].x |= kCFilter;
            const int4 v = C.ce[c];
            e = (e & 1) ? v.w : v.y;
        }
    }
}

int NextContactEdge(const HWorld& W, int e)
{
    const int4 v = W.contacts.ce[e >> 1];
    return (e & 1) ? v.w : v.y;
}

// b2World::DestroyBody (Dynamics/b2World.cpp:133-212)
void DestroyBodyHost(HWorld& W, int bi, Calls& calls)
{
    for (int e = W.bodies[bi].jointList; e != kNullIdx;) {
        const int jn = e >> 1;
        e = W.joints[jn].eNext[e & 1];
        calls.insert(calls.end(), {0, jn, 0});
        DestroyJointHost(W, jn);
        W.bodies[bi].jointList = e;
    }
    W.bodies[bi].jointList = kNullIdx;
    if (W.hasState)
        for (int e = W.bodies[bi].contactList; e != kNullIdx;) {
            const int c = e >> 1;
            e = NextContactEdge(W, e);
            DestroyContactHost(W, c, calls);
        }
    W.bodies[bi].contactList = kNullIdx;
    for (int f = W.bodies[bi].fixtureList; f != kNullIdx;) {
        HFixture& fx = W.fixtures[f];
        const int next = fx.next;
        if (fx.shape.chain != 2) calls.insert(calls.end(), {1, f, 0});  // a chain is one b2Fixture
        if (fx.proxyId != kNullIdx) FreeProxy(W, fx.proxyId);
        fx.proxyId = kNullIdx;
        fx.body = kNullIdx;
        fx.next = kNullIdx;
        W.bodies[bi].fixtureList = next;
        f = next;
    }
    if (W.bodyList == bi) {
        W.bodyList = W.bodies[bi].next;
    } else {
        for (int b = W.bodyList; b != kNullIdx; b = W.bodies[b].next)
            if (W.bodies[b].next == bi) { W.bodies[b].next = W.bodies[bi].next; break; }
    }
    HBody dead;
    dead.alive = false;
    dead.xf.p = V(0.0f, 0.0f);
    dead.xf.q.s = 0.0f;
    dead.xf.q.c = 0.0f;
    dead.sw.localCenter = V(0.0f, 0.0f);
    dead.sw.c0 = dead.sw.c = V(0.0f, 0.0f);
    dead.sw.a0 = dead.sw.a = dead.sw.alpha0 = 0.0f;
    dead.gravScale = 0.0f;
    W.bodies[bi] = dead;
}

// b2Body::DestroyFixture (Dynamics/b2Body.cpp:216-281); a chain (its first child) goes whole
void DestroyFixtureHost(HWorld& W, int f, Calls& calls)
{
    const int bi = W.fixtures[f].body;
    int last = f;
    if (W.fixtures[f].shape.type == kEdge && W.fixtures[f].shape.chain == 1)
        while (last + 1 < (int)W.fixtures.size() && W.fixtures[last + 1].body == bi &&
               W.fixtures[last + 1].shape.type == kEdge && W.fixtures[last + 1].shape.chain == 2)
            ++last;
    auto mine = [&](int id) { return id >= f && id <= last; };
    int* node = &W.bodies[bi].fixtureList;
    while (*node != kNullIdx && !mine(*node)) node = &W.fixtures[*node].next;
    int after = *node;
    while (after != kNullIdx && mine(after)) after = W.fixtures[after].next;
    if (*node != kNullIdx) *node = after;
    if (W.hasState)
        for (int e = W.bodies[bi].contactList; e != kNullIdx;) {
            const int c = e >> 1;
            e = NextContactEdge(W, e);
            const int4 info = W.contacts.ci[c];
            if (mine(info.y) || mine(info.z)) DestroyContactHost(W, c, calls);
        }
    for (int id = f; id <= last; ++id) {
        HFixture& fx = W.fixtures[id];
        if ((W.bodies[bi].flags & kBActive) && fx.proxyId != kNullIdx) FreeProxy(W, fx.proxyId);
        fx.proxyId = kNullIdx;
        fx.body = kNullIdx;
        fx.next = kNullIdx;
    }
    ResetMassData(W, bi);
}

gb_status Finish(const Calls& calls, int* out, int cap, int* n_calls)
{
    const int n = (int)calls.size() / 3;
    if (out)
        for (int i = 0; i < 3 * std::min(n, std::max(cap, 0)); ++i) out[i] = calls[i];
    if (n_calls) *n_calls = n;
    return GB_OK;
}

} // namespace

extern "C" {

gb_status gb_world_create(int n_worlds, const gb_world_def* defs, gb_world** out)
{
    if (!out || n_worlds <= 0 || !defs) return GB_ERR_INVALID;
    *out = nullptr;
    gb_world* g = new (std::nothrow) gb_world();
    if (!g) return GB_ERR_CAPACITY;
    g->worlds.resize(n_worlds);
    for (int i = 0; i < n_worlds; ++i) g->worlds[i].def = defs[i];
    // The stream is created at the first upload, so building a world needs no device.
    *out = g;
    return GB_OK;
}

gb_status gb_world_destroy(gb_world* g)
{
    if (!g) return GB_ERR_INVALID;
    if (g->stream) cudaStreamSynchronize(g->stream);
    for (int i = 0; i < kMaxClasses; ++i)
        if (g->side[i]) cudaStreamSynchronize(g->side[i]);
    ReleaseTransferResources(g);
    FreeDevice(g);
    ReleaseLaunchResources(g);
    FreeLog(g);
    if (g->dEdits) cudaFree(g->dEdits);
    if (g->dContactEdits) cudaFree(g->dContactEdits);
    FreeFilter(g);
    if (g->ownStream && g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return GB_OK;
}

static_assert(sizeof(gb_body_edit) == sizeof(BodyEdit), "gb_body_edit and its device copy share a layout");

gb_status gb_body_edits(gb_world* g, int n, const gb_body_edit* edits)
{
    if (!g || n < 0 || (n > 0 && !edits)) return GB_ERR_INVALID;
    if (n == 0) return GB_OK;
    for (int i = 0; i < n; ++i) {
        const gb_body_edit& e = edits[i];
        if (e.world < 0 || e.world >= (int)g->worlds.size()) return GB_ERR_INVALID;
        if (e.op < 0 || e.op >= kEditOps) return GB_ERR_INVALID;
        const HWorld& W = g->worlds[e.world];
        if (e.op == kEditMouseTarget) {
            // body is the joint index; only a mouse joint has a target
            if (e.body < 0 || e.body >= (int)W.joints.size() || W.joints[e.body].type != kJointMouse) return GB_ERR_INVALID;
        } else if (e.body < 0 || e.body >= (int)W.bodies.size()) {
            return GB_ERR_INVALID;
        }
    }
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    if (g->editCap < n) {
        // freeing waits for the device, so an earlier call's edits are no longer read
        if (g->dEdits) GB_CUDA(cudaFree(g->dEdits));
        g->dEdits = nullptr;
        g->editCap = 0;
        GB_CUDA(cudaMalloc(&g->dEdits, (size_t)n * sizeof(BodyEdit)));
        g->editCap = n;
    }
    // from pageable memory the copy has left the caller's array when the call returns; stream order
    // keeps an earlier call's kernel ahead of this copy
    GB_CUDA(cudaMemcpyAsync(g->dEdits, edits, (size_t)n * sizeof(BodyEdit), cudaMemcpyHostToDevice, g->stream));
    GB_CUDA(b2gLaunchBodyEdits(g->batch, g->dEdits, n, g->stream));
    return GB_OK;
}

gb_status gb_create_bodies(gb_world* g, int w, int n, const int* type, const float* f, const int* flags, int* out_ids)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    for (int i = 0; i < n; ++i)
        if ((s = CreateBody(g->worlds[w], type[i], f + 9 * i, flags[i], out_ids ? out_ids + i : nullptr)) != GB_OK) return s;
    return GB_OK;
}

gb_status gb_create_fixtures(gb_world* g, int w, int n, const int* body, const int* shape_type, const float* shape,
                             const int* shape_n, const float* mat, const int* filt, int* out_ids)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    for (int i = 0; i < n; ++i)
        if ((s = CreateFixture(g->worlds[w], body[i], shape_type[i], shape + 16 * i, shape_n[i], mat + 3 * i, filt + 4 * i,
                               out_ids ? out_ids + i : nullptr)) != GB_OK)
            return s;
    return GB_OK;
}

gb_status gb_create_chain(gb_world* g, int w, int body, const float* xy, int count, int loop, const float* prev_next,
                          int ghost_flags, const float* mat, const int* filt, int* first_id)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    if (!xy || !mat || !filt || count < (loop ? 3 : 2) || (!loop && ghost_flags != 0 && !prev_next)) return GB_ERR_INVALID;
    // b2ChainShape::CreateLoop / CreateChain (Collision/Shapes/b2ChainShape.cpp:36-80): a loop repeats
    // its first vertex and takes the last and second vertices as its ghosts
    std::vector<Vec2> v((size_t)count + (loop ? 1 : 0));
    for (int i = 0; i < count; ++i) v[i] = V(xy[2 * i], xy[2 * i + 1]);
    Vec2 prevV = V(0.0f, 0.0f), nextV = V(0.0f, 0.0f);
    bool hasPrev = false, hasNext = false;
    if (loop) {
        v[count] = v[0];
        prevV = v[count - 1]; nextV = v[1];
        hasPrev = hasNext = true;
    } else {
        if (ghost_flags & 1) { prevV = V(prev_next[0], prev_next[1]); hasPrev = true; }
        if (ghost_flags & 2) { nextV = V(prev_next[2], prev_next[3]); hasNext = true; }
    }
    // b2ChainShape::GetChildEdge (b2ChainShape.cpp:112-142) for each child, one fixture each
    const int m = (int)v.size();
    for (int i = 0; i < m - 1; ++i) {
        const Vec2 v0 = i > 0 ? v[i - 1] : prevV, v3 = i < m - 2 ? v[i + 2] : nextV;
        const bool h0 = i > 0 || hasPrev, h3 = i < m - 2 || hasNext;
        float rec[16] = {v[i].x, v[i].y, v[i + 1].x, v[i + 1].y, v0.x, v0.y, v3.x, v3.y, h0 ? 1.0f : 0.0f,
                         h3 ? 1.0f : 0.0f, i == 0 ? 1.0f : 2.0f};
        int id = -1;
        if ((s = CreateFixture(g->worlds[w], body, 1, rec, 2, mat, filt, &id)) != GB_OK) return s;
        if (i == 0 && first_id) *first_id = id;
    }
    return GB_OK;
}

gb_status gb_create_revolute_joints(gb_world* g, int w, int n, const int* a, const int* b, const float* f,
                                    const int* flags, int* out_ids)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    for (int i = 0; i < n; ++i)
        if ((s = CreateJoint(g->worlds[w], kJointRevolute, a[i], b[i], f + 9 * i, flags[i], out_ids ? out_ids + i : nullptr)) != GB_OK)
            return s;
    return GB_OK;
}

gb_status gb_create_joints(gb_world* g, int w, int n, const int* type, const int* a, const int* b, const float* f,
                           const int* flags, int* out_ids)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    if (n > 0 && (!type || !a || !b || !f || !flags)) return GB_ERR_INVALID;
    for (int i = 0; i < n; ++i)
        if ((s = CreateJoint(g->worlds[w], type[i], a[i], b[i], f + GB_JOINT_FLOATS * i, flags[i], out_ids ? out_ids + i : nullptr)) != GB_OK)
            return s;
    return GB_OK;
}

gb_status gb_build_world(gb_world* g, int w, int nb, const int* body_type, const float* body_f, const int* body_flags,
                         int nf, const int* fix_body, const int* fix_type, const float* fix_shape, const int* fix_n,
                         const float* fix_mat, const int* fix_filt, int nj, const int* joint_type, const int* joint_a,
                         const int* joint_b, const float* joint_f, const int* joint_flags)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    HWorld& W = g->worlds[w];
    const int base = (int)W.bodies.size();
    int fi = 0;
    for (int b = 0; b < nb; ++b) {
        if ((s = CreateBody(W, body_type[b], body_f + 9 * b, body_flags[b], nullptr)) != GB_OK) return s;
        while (fi < nf && fix_body[fi] == b) {
            if ((s = CreateFixture(W, base + b, fix_type[fi], fix_shape + 16 * fi, fix_n[fi], fix_mat + 3 * fi,
                                   fix_filt + 4 * fi, nullptr)) != GB_OK)
                return s;
            ++fi;
        }
    }
    if (fi != nf) return GB_ERR_INVALID;
    for (int j = 0; j < nj; ++j)
        if ((s = CreateJoint(W, joint_type ? joint_type[j] : kJointRevolute, base + joint_a[j], base + joint_b[j],
                             joint_f + GB_JOINT_FLOATS * j, joint_flags[j], nullptr)) != GB_OK)
            return s;
    return GB_OK;
}

gb_status gb_world_upload(gb_world* g)
{
    if (!g) return GB_ERR_INVALID;
    return Upload(g);
}

gb_status gb_world_step_begin(gb_world* g, float dt, int vi, int pi)
{
    if (!g || vi < 0 || pi < 0 || g->splitOpen || g->filterFn) return GB_ERR_INVALID;
    gb_status s = TreeSync(g);
    if (s == GB_OK) s = Upload(g);
    if (s != GB_OK) return s;
    StepParams P = MakeParams(g, dt, vi, pi);
    P.phase = 1;
    s = LaunchPlanStep(g, P, g->plan);
    if (s != GB_OK) return s;
    g->splitOpen = true;
    g->locked = true;  // as inside b2World::Step: no creation or destruction until the step ends
    g->splitDt = dt;
    g->splitVi = vi;
    g->splitPi = pi;
    return GB_OK;
}

gb_status gb_contact_edits(gb_world* g, int n, const gb_contact_edit* edits)
{
    static_assert(sizeof(gb_contact_edit) == sizeof(ContactEdit), "gb_contact_edit mirrors the device record");
    if (!g || n < 0 || (n > 0 && !edits) || !g->splitOpen) return GB_ERR_INVALID;
    if (n == 0) return GB_OK;
    if (n > g->contactEditCap) {
        if (g->dContactEdits) cudaFree(g->dContactEdits);
        g->dContactEdits = nullptr;
        g->contactEditCap = 0;
        GB_CUDA(cudaMalloc(&g->dContactEdits, n * sizeof(ContactEdit)));
        g->contactEditCap = n;
    }
    GB_CUDA(cudaMemcpyAsync(g->dContactEdits, edits, n * sizeof(ContactEdit), cudaMemcpyHostToDevice, g->stream));
    GB_CUDA(b2gLaunchContactEdits(g->batch, g->dContactEdits, n, g->stream));
    GB_CUDA(cudaStreamSynchronize(g->stream));  // the host array may go once the call returns
    return GB_OK;
}

gb_status gb_world_step_end(gb_world* g)
{
    if (!g || !g->splitOpen) return GB_ERR_INVALID;
    StepParams P = MakeParams(g, g->splitDt, g->splitVi, g->splitPi);
    P.phase = 2;
    g->splitOpen = false;
    g->locked = false;
    return LaunchPlanStep(g, P, g->plan);
}

gb_status gb_world_step(gb_world* g, float dt, int vi, int pi)
{
    if (!g || vi < 0 || pi < 0 || g->splitOpen) return GB_ERR_INVALID;
    gb_status s = TreeSync(g);
    if (s == GB_OK) s = Upload(g);
    if (s != GB_OK) return s;
    if (g->recoverAttempts > 0) return RecoveringStep(g, dt, vi, pi);
    const StepParams P = MakeParams(g, dt, vi, pi);
    if (g->filterFn) return FilteredStep(g, P);
    if (g->tuneIndex >= 0) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        GB_CUDA(cudaStreamIsCapturing(g->stream, &cs));
        if (cs == cudaStreamCaptureStatusNone) return TunedStep(g, P);
    }
    return LaunchPlanStep(g, P, g->plan);
}

gb_status gb_world_set_contact_filter(gb_world* g, gb_should_collide_fn fn, void* user)
{
    if (!g || g->splitOpen) return GB_ERR_INVALID;
    ReleaseGraph(g);
    g->filterFn = fn;
    g->filterUser = user;
    if (!fn) {
        FreeFilter(g);
        AttachFilter(g);
        return GB_OK;
    }
    for (const HWorld& W : g->worlds)
        if ((int)W.fixtures.size() >= (1 << 20) || g->worlds.size() >= (1u << 23)) return GB_ERR_CAPACITY;
    if (!g->dFilterMiss) GB_CUDA(cudaMalloc(&g->dFilterMiss, sizeof(int)));
    gb_status s = BuildFilterTable(g, 4096, {}, {});
    if (s != GB_OK) return s;
    AttachFilter(g);
    return GB_OK;
}

gb_status gb_world_refilter(gb_world* g, int w, int fixture)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || !g->filterFn) return GB_ERR_INVALID;
    std::vector<unsigned long long> keys((size_t)g->filterCap);
    std::vector<int> vals((size_t)g->filterCap);
    GB_CUDA(cudaMemcpy(keys.data(), g->dFilterKeys, g->filterCap * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    GB_CUDA(cudaMemcpy(vals.data(), g->dFilterVals, g->filterCap * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<unsigned long long> kk;
    std::vector<int> vv;
    for (int i = 0; i < g->filterCap; ++i) {
        if (keys[i] == ~0ull) continue;
        const int kw = (int)(keys[i] >> 40), fA = (int)((keys[i] >> 20) & 0xFFFFF), fB = (int)(keys[i] & 0xFFFFF);
        if (kw == w && (fA == fixture || fB == fixture)) continue;  // decided again when next met
        kk.push_back(keys[i]);
        vv.push_back(vals[i]);
    }
    gb_status s = BuildFilterTable(g, g->filterCap, kk, vv);
    if (s != GB_OK) return s;
    AttachFilter(g);
    ReleaseGraph(g);
    return GB_OK;
}

gb_status gb_world_filter_stats(gb_world* g, long long* replays, int* verdicts)
{
    if (!g) return GB_ERR_INVALID;
    if (replays) *replays = g->filterReplays;
    if (verdicts) *verdicts = g->filterUsed;
    return GB_OK;
}

gb_status gb_world_graph_step(gb_world* g, float dt, int vi, int pi)
{
    if (!g || vi < 0 || pi < 0 || g->splitOpen) return GB_ERR_INVALID;
    if (g->filterFn) return gb_world_step(g, dt, vi, pi);  // a filtered step may run again: no graph
    if (g->recoverAttempts > 0) return gb_world_step(g, dt, vi, pi);  // so may a recovering one
    if (g->tuneIndex >= 0) return gb_world_step(g, dt, vi, pi);  // tuning steps are timed one by one
    gb_status s = TreeSync(g);
    if (s == GB_OK) s = Upload(g);
    if (s != GB_OK) return s;
    const bool reuse = g->graph && g->graphDt == dt && g->graphVi == vi && g->graphPi == pi &&
                       g->graphSolver == g->solver && g->graphTol == g->tolerance &&
                       g->graphMeasure == g->measureResidual && g->graphWarm == g->warmMode &&
                       g->graphLog == g->logX && SamePlan(g->graphPlan, g->plan);
    if (!reuse) {
        ReleaseGraph(g);
        if (g->plan.size() > 1) {
            s = EnsureSideStreams(g, (int)g->plan.size());
            if (s != GB_OK) return s;
        }
        const StepParams P = MakeParams(g, dt, vi, pi);
        GB_CUDA(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
        s = LaunchPlanStep(g, P, g->plan);
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(g->stream, &graph);
        if (s != GB_OK) { if (graph) cudaGraphDestroy(graph); return s; }
        GB_CUDA(ec);
        // node priorities from the capture (the class pipelines' stream priorities) are kept
        const cudaError_t ei = cudaGraphInstantiate(&g->graph, graph, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(graph);
        GB_CUDA(ei);
        g->graphDt = dt; g->graphVi = vi; g->graphPi = pi; g->graphSolver = g->solver;
        g->graphTol = g->tolerance; g->graphMeasure = g->measureResidual; g->graphPlan = g->plan;
        g->graphWarm = g->warmMode; g->graphLog = g->logX;
    }
    GB_CUDA(cudaGraphLaunch(g->graph, g->stream));
    return GB_OK;
}

gb_status gb_world_autotune(gb_world* g, int steps_per_candidate)
{
    if (!g || steps_per_candidate < 1 || steps_per_candidate > 64) return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    for (cudaEvent_t e : g->tuneEvents) cudaEventDestroy(e);
    g->tuneEvents.clear();
    g->candidates = CandidatePlans(g);
    g->candidateMs.assign(g->candidates.size(), 0.0f);
    const size_t n = 2 * g->candidates.size() * (size_t)steps_per_candidate;
    for (size_t i = 0; i < n; ++i) {
        cudaEvent_t e = nullptr;
        GB_CUDA(cudaEventCreate(&e));
        g->tuneEvents.push_back(e);
    }
    g->tuneSteps = steps_per_candidate;
    g->tuneIndex = 0;
    g->tuneRep = 0;
    return GB_OK;
}

gb_status gb_world_launch_plan(gb_world* g, int* classes, int cap, int* n_classes, float* candidate_ms, int ms_cap,
                               int* n_candidates)
{
    if (!g) return GB_ERR_INVALID;
    if (n_classes) *n_classes = (int)g->plan.size();
    if (classes)
        for (int i = 0; i < (int)g->plan.size() && i < cap; ++i) {
            const LaunchClass& c = g->plan[i];
            classes[5 * i] = c.first; classes[5 * i + 1] = c.count; classes[5 * i + 2] = c.threads;
            classes[5 * i + 3] = c.rows; classes[5 * i + 4] = c.contacts;
        }
    const int nc = g->tuneIndex < 0 ? (int)g->candidateMs.size() : 0;
    if (n_candidates) *n_candidates = nc;
    if (candidate_ms)
        for (int i = 0; i < nc && i < ms_cap; ++i) candidate_ms[i] = g->candidateMs[i];
    return GB_OK;
}

gb_status gb_world_set_launch_plan(gb_world* g, const int* classes, int n)
{
    if (!g || !classes || n < 1 || n > kMaxClasses) return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    LaunchPlan plan;
    int next = 0;
    for (int i = 0; i < n; ++i) {
        LaunchClass c{classes[5 * i], classes[5 * i + 1], classes[5 * i + 2], classes[5 * i + 3], classes[5 * i + 4]};
        const size_t smem = (2 * (size_t)std::max(c.rows, 0) + std::max(c.contacts, 0)) * sizeof(float4);
        if (c.first != next || c.count < 1 || c.threads < 32 || c.threads > 512 || c.threads % 32 != 0 ||
            c.rows < 0 || c.contacts < 0 || smem > 48 * 1024)
            return GB_ERR_INVALID;
        next += c.count;
        plan.push_back(c);
    }
    if (next != (int)g->schedule.size()) return GB_ERR_INVALID;
    g->plan = plan;
    g->tuneIndex = -1;
    return GB_OK;
}

gb_status gb_world_sync(gb_world* g)
{
    if (!g) return GB_ERR_INVALID;
    if (!g->onDevice) return GB_OK;
    GB_CUDA(cudaStreamSynchronize(g->stream));
    if (g->upStream) GB_CUDA(cudaStreamSynchronize(g->upStream));
    if (g->downStream) GB_CUDA(cudaStreamSynchronize(g->downStream));
    const int nw = (int)g->worlds.size();
    std::vector<WorldState> st(nw);
    GB_CUDA(cudaMemcpy(st.data(), g->batch.state, nw * sizeof(WorldState), cudaMemcpyDeviceToHost));
    int err = 0;
    for (const WorldState& s : st) err |= s.error;
    if (err & kErrCapacity) return GB_ERR_CAPACITY;
    if (err & kErrTimeout) return GB_ERR_TIMEOUT;
    if (err & kErrInvalid) return GB_ERR_INVALID;
    return GB_OK;
}

// b2World::SetGravity, SetAllowSleeping, SetWarmStarting, SetContinuousPhysics, SetSubStepping and
// SetAutoClearForces (Dynamics/b2World.h:145-217, b2World.cpp:370-385) between steps: turning sleep
// off wakes every body of the world's body list (b2Body::SetAwake(true): awake, sleep time 0).
gb_status gb_world_set_settings(gb_world* g, int w, const gb_world_def* def, int auto_clear_forces)
{
    if (!g || !def || w < 0 || w >= (int)g->worlds.size() || g->locked) return GB_ERR_INVALID;
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    HWorld& W = g->worlds[w];
    if (W.def.allow_sleep && !def->allow_sleep) {
        int guard = 0;
        for (int b = W.bodyList; b != kNullIdx && guard <= (int)W.bodies.size(); b = W.bodies[b].next, ++guard) {
            HBody& B = W.bodies[b];
            if ((B.flags & kBAwake) == 0) {
                B.flags |= kBAwake;
                B.sleepTime = 0.0f;
            }
        }
    }
    W.def = *def;
    W.autoClear = auto_clear_forces != 0;
    return GB_OK;
}

// b2World::ClearForces (Dynamics/b2World.cpp:967-974): every body's force and torque zeroed.
gb_status gb_world_clear_forces(gb_world* g, int w)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || g->locked) return GB_ERR_INVALID;
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    for (HBody& B : g->worlds[w].bodies) {
        B.force = V(0.0f, 0.0f);
        B.torque = 0.0f;
    }
    return GB_OK;
}

gb_status gb_world_set_recovery(gb_world* g, int attempts)
{
    if (!g || attempts < 0 || attempts > 30 || g->splitOpen) return GB_ERR_INVALID;
    g->recoverAttempts = attempts;
    if (attempts == 0) {
        for (void* p : g->recoverShadow) cudaFree(p);
        g->recoverShadow.clear();
    }
    return GB_OK;
}

gb_status gb_world_recoveries(gb_world* g, long long* retries)
{
    if (!g || !retries) return GB_ERR_INVALID;
    *retries = g->recoveries;
    return GB_OK;
}

gb_status gb_world_set_limits(gb_world* g, int contact_capacity, int max_toi_events)
{
    if (!g || contact_capacity < 0 || max_toi_events < 1) return GB_ERR_INVALID;
    if (contact_capacity > 0 && g->onDevice) return GB_ERR_INVALID;
    g->contactCapLimit = contact_capacity;
    if (g->maxToiEvents != max_toi_events) ReleaseGraph(g);
    g->maxToiEvents = max_toi_events;
    return GB_OK;
}

gb_status gb_world_set_solver(gb_world* g, int solver, float tolerance, int measure_residual)
{
    if (!g || (solver != kSolverPlain && solver != kSolverColoured) || !(tolerance >= 0.0f)) return GB_ERR_INVALID;
    g->solver = solver;
    g->tolerance = tolerance;
    g->measureResidual = measure_residual ? 1 : 0;
    return GB_OK;
}

gb_status gb_world_set_warm_start(gb_world* g, gb_mlp* mlp, int mode)
{
    if (!g || mode < kWarmReference || mode > kWarmLearnedAll || (mode != kWarmReference && !mlp)) return GB_ERR_INVALID;
    g->warmMode = mode;
    g->mlp = mode != kWarmReference ? b2gMlpView(mlp) : MlpView{};
    ReleaseGraph(g);  // a captured step holds the previous network's view
    return GB_OK;
}

gb_status gb_world_query_aabb(gb_world* g, int w, int n, const float* aabbs, int* offsets, int* fixtures, int cap,
                             int* total)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || n < 0 || !offsets || !total || cap < 0 || (n > 0 && !aabbs))
        return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    *total = 0;
    offsets[0] = 0;
    if (n == 0) return GB_OK;
    float4* dBoxes = nullptr;
    int *dCounts = nullptr, *dOffsets = nullptr, *dFill = nullptr;
    std::vector<int> counts(n);
    cudaError_t e = cudaMalloc(&dBoxes, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&dCounts, n * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&dOffsets, (n + 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dBoxes, aabbs, n * sizeof(float4), cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = b2gLaunchQueryAabb(g->batch, w, dBoxes, n, nullptr, dCounts, nullptr, 0, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts.data(), dCounts, n * sizeof(int), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) {
        for (int i = 0; i < n; ++i) offsets[i + 1] = offsets[i] + counts[i];
        *total = offsets[n];
        const int m = std::min(*total, cap);
        if (m > 0 && fixtures) {
            e = cudaMalloc(&dFill, m * sizeof(int));
            if (e == cudaSuccess) e = cudaMemcpyAsync(dOffsets, offsets, (n + 1) * sizeof(int), cudaMemcpyHostToDevice, g->stream);
            if (e == cudaSuccess) e = b2gLaunchQueryAabb(g->batch, w, dBoxes, n, dOffsets, dCounts, dFill, m, g->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(fixtures, dFill, m * sizeof(int), cudaMemcpyDeviceToHost, g->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
        }
    }
    cudaFree(dBoxes); cudaFree(dCounts); cudaFree(dOffsets); cudaFree(dFill);
    GB_CUDA(e);
    return *total > cap ? GB_ERR_CAPACITY : GB_OK;
}

gb_status gb_world_raycast_all(gb_world* g, int w, const float* ray, int* fixtures, float* hits, int cap, int* n)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || !ray || !n || cap < 0 || (cap > 0 && (!fixtures || !hits)))
        return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    *n = 0;
    const int nf = g->desc[w].fixCount;
    if (nf == 0) return GB_OK;
    float4* dHits = nullptr;
    int* dCount = nullptr;
    cudaError_t e = cudaMalloc(&dHits, nf * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&dCount, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(dCount, 0, sizeof(int), g->stream);
    if (e == cudaSuccess)
        e = b2gLaunchRayCastAll(g->batch, w, nf, make_float4(ray[0], ray[1], ray[2], ray[3]), dHits, dCount, nf,
                                g->stream);
    int count = 0;
    std::vector<float4> h;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&count, dCount, sizeof(int), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess && count > 0) {
        h.resize(count);
        e = cudaMemcpy(h.data(), dHits, count * sizeof(float4), cudaMemcpyDeviceToHost);
    }
    cudaFree(dHits);
    cudaFree(dCount);
    GB_CUDA(e);
    // fixture order: the order the reference's callbacks would see is its tree's, which is not kept
    std::sort(h.begin(), h.end(), [](const float4& a, const float4& b) { return __float_as_int_host(a.x) < __float_as_int_host(b.x); });
    const Vec2 p1 = V(ray[0], ray[1]), p2 = V(ray[2], ray[3]);
    for (int k = 0; k < count && k < cap; ++k) {
        const float f = h[k].y;
        const Vec2 pt = (1.0f - f) * p1 + f * p2;
        fixtures[k] = __float_as_int_host(h[k].x);
        hits[5 * k] = f;
        hits[5 * k + 1] = pt.x;
        hits[5 * k + 2] = pt.y;
        hits[5 * k + 3] = h[k].z;
        hits[5 * k + 4] = h[k].w;
    }
    *n = count;
    return count > cap ? GB_ERR_CAPACITY : GB_OK;
}

gb_status gb_world_get_profile(gb_world* g, int w, float* ms)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || !ms) return GB_ERR_INVALID;
    for (int k = 0; k < 8; ++k) ms[k] = 0.0f;
    if (!g->onDevice) return GB_OK;
    GB_CUDA(cudaStreamSynchronize(g->stream));
    WorldState st;
    GB_CUDA(cudaMemcpy(&st, g->batch.state + w, sizeof(WorldState), cudaMemcpyDeviceToHost));
    int dev = 0, khz = 0;
    GB_CUDA(cudaGetDevice(&dev));
    GB_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
    const double perMs = khz > 0 ? (double)khz : 1.0;
    auto c = [&](int k) { return (double)st.cyc[k]; };
    // b2Profile (Box2D/Dynamics/b2TimeStep.h:27-37): step, collide, solve, solveInit, solveVelocity,
    // solvePosition, broadphase (fixture sync and pair finding after the islands), solveTOI
    const double v[8] = {c(7), c(0) + c(1), c(2) + c(3) + c(4) + c(5), c(8), c(9), c(11), c(4) + c(5), c(6)};
    for (int k = 0; k < 8; ++k) ms[k] = (float)(v[k] / perMs);
    return GB_OK;
}

gb_status gb_world_raycast(gb_world* g, int w, int n, const float* rays, int* fixture, float* hit)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || n < 0 || (n > 0 && (!rays || !fixture || !hit)))
        return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    if (n == 0) return GB_OK;
    float4* dRays = nullptr;
    int* dFix = nullptr;
    float* dHit = nullptr;
    cudaError_t e = cudaMalloc(&dRays, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&dFix, n * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&dHit, 5 * (size_t)n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dRays, rays, n * sizeof(float4), cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = b2gLaunchRayCast(g->batch, w, dRays, n, dFix, dHit, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fixture, dFix, n * sizeof(int), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hit, dHit, 5 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cudaFree(dRays); cudaFree(dFix); cudaFree(dHit);
    GB_CUDA(e);
    return GB_OK;
}

gb_status gb_world_set_events(gb_world* g, int enable)
{
    if (!g) return GB_ERR_INVALID;
    const bool on = enable != 0;
    if (on == g->eventsEnabled) return GB_OK;
    g->eventsEnabled = on;
    // the log is sized with the device columns: reallocate them (the state is preserved)
    g->hostDirty = true;
    return Upload(g);
}

gb_status gb_world_read_events(gb_world* g, int w, int* records, float* impulses, int cap, int* n)
{
    if (!g || !n || cap < 0 || w < 0 || w >= (int)g->worlds.size()) return GB_ERR_INVALID;
    *n = 0;
    if (!g->onDevice || !g->eventsEnabled) return GB_OK;
    GB_CUDA(cudaStreamSynchronize(g->stream));
    WorldState st;
    GB_CUDA(cudaMemcpy(&st, g->batch.state + w, sizeof(WorldState), cudaMemcpyDeviceToHost));
    const int count = std::min(st.eventCount, 4 * g->desc[w].contactCap);
    *n = count;
    const int m = std::min(count, cap);
    if (m > 0) {
        std::vector<int4> raw(2 * (size_t)m);
        GB_CUDA(cudaMemcpy(raw.data(), g->batch.evLog + 8 * (size_t)g->desc[w].contactBase, raw.size() * sizeof(int4),
                           cudaMemcpyDeviceToHost));
        for (int i = 0; i < m; ++i) {
            if (records) {
                records[4 * i] = raw[2 * i].x; records[4 * i + 1] = raw[2 * i].y;
                records[4 * i + 2] = raw[2 * i].z; records[4 * i + 3] = raw[2 * i].w;
            }
            if (impulses) std::memcpy(impulses + 4 * (size_t)i, &raw[2 * i + 1], 4 * sizeof(float));
        }
    }
    return st.eventsDropped ? GB_ERR_CAPACITY : GB_OK;
}

gb_status gb_world_set_contact_log(gb_world* g, int capacity)
{
    if (!g || capacity < 0) return GB_ERR_INVALID;
    if (g->stream) GB_CUDA(cudaStreamSynchronize(g->stream));
    FreeLog(g);
    if (capacity == 0) return GB_OK;
    GB_CUDA(cudaMalloc(&g->logX, (size_t)capacity * 14 * sizeof(float)));
    GB_CUDA(cudaMalloc(&g->logT, (size_t)capacity * 2 * sizeof(float)));
    GB_CUDA(cudaMalloc(&g->logCount, sizeof(int)));
    GB_CUDA(cudaMemset(g->logCount, 0, sizeof(int)));
    g->logCap = capacity;
    return GB_OK;
}

gb_status gb_world_read_contact_log(gb_world* g, float* x, float* t, int cap, int* n)
{
    if (!g || !n || cap < 0) return GB_ERR_INVALID;
    *n = 0;
    if (!g->logCount) return GB_OK;
    if (g->stream) GB_CUDA(cudaStreamSynchronize(g->stream));
    int count = 0;
    GB_CUDA(cudaMemcpy(&count, g->logCount, sizeof(int), cudaMemcpyDeviceToHost));
    const int m = std::min(std::min(count, g->logCap), cap);
    if (m > 0 && x) GB_CUDA(cudaMemcpy(x, g->logX, (size_t)m * 14 * sizeof(float), cudaMemcpyDeviceToHost));
    if (m > 0 && t) GB_CUDA(cudaMemcpy(t, g->logT, (size_t)m * 2 * sizeof(float), cudaMemcpyDeviceToHost));
    GB_CUDA(cudaMemset(g->logCount, 0, sizeof(int)));
    *n = m;
    return count > g->logCap ? GB_ERR_CAPACITY : GB_OK;
}

gb_status gb_world_solver_stats(gb_world* g, int* colours, int* vel_iters, float* residual)
{
    if (!g) return GB_ERR_INVALID;
    const int nw = (int)g->worlds.size();
    if (!g->onDevice) {
        for (int i = 0; i < nw; ++i) {
            if (colours) colours[i] = 0;
            if (vel_iters) vel_iters[i] = 0;
            if (residual) residual[i] = 0.0f;
        }
        return GB_OK;
    }
    GB_CUDA(cudaStreamSynchronize(g->stream));
    std::vector<WorldState> st(nw);
    GB_CUDA(cudaMemcpy(st.data(), g->batch.state, nw * sizeof(WorldState), cudaMemcpyDeviceToHost));
    for (int i = 0; i < nw; ++i) {
        if (colours) colours[i] = st[i].colours;
        if (vel_iters) vel_iters[i] = st[i].velIters;
        if (residual) residual[i] = st[i].residual;
    }
    return GB_OK;
}

gb_status gb_world_contact_stats(gb_world* g, float* max_penetration)
{
    if (!g || !max_penetration) return GB_ERR_INVALID;
    const int nw = (int)g->worlds.size();
    if (!g->onDevice) {
        for (int i = 0; i < nw; ++i) max_penetration[i] = 0.0f;
        return GB_OK;
    }
    GB_CUDA(cudaStreamSynchronize(g->stream));
    std::vector<WorldState> st(nw);
    GB_CUDA(cudaMemcpy(st.data(), g->batch.state, nw * sizeof(WorldState), cudaMemcpyDeviceToHost));
    for (int i = 0; i < nw; ++i) max_penetration[i] = st[i].maxPenetration;
    return GB_OK;
}

gb_status gb_world_warm_stats(gb_world* g, int* learned_islands, int* vel_iters_sum)
{
    if (!g) return GB_ERR_INVALID;
    const int nw = (int)g->worlds.size();
    if (!g->onDevice) {
        for (int i = 0; i < nw; ++i) {
            if (learned_islands) learned_islands[i] = 0;
            if (vel_iters_sum) vel_iters_sum[i] = 0;
        }
        return GB_OK;
    }
    GB_CUDA(cudaStreamSynchronize(g->stream));
    std::vector<WorldState> st(nw);
    GB_CUDA(cudaMemcpy(st.data(), g->batch.state, nw * sizeof(WorldState), cudaMemcpyDeviceToHost));
    for (int i = 0; i < nw; ++i) {
        if (learned_islands) learned_islands[i] = st[i].warmLearned;
        if (vel_iters_sum) vel_iters_sum[i] = st[i].velItersSum;
    }
    return GB_OK;
}

gb_status gb_world_set_stream(gb_world* g, void* stream)
{
    if (!g) return GB_ERR_INVALID;
    if (g->stream) GB_CUDA(cudaStreamSynchronize(g->stream));
    ReleaseTransferResources(g);
    if (g->ownStream && g->stream) cudaStreamDestroy(g->stream);
    if (stream) { g->stream = static_cast<cudaStream_t>(stream); g->ownStream = false; }
    else {
        GB_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
        g->ownStream = true;
    }
    return GB_OK;
}

gb_status gb_world_counts(gb_world* g, int w, int* bodies, int* fixtures, int* contacts, int* joints)
{
    if (!g || w < 0 || w >= (int)g->worlds.size()) return GB_ERR_INVALID;
    HWorld& W = g->worlds[w];
    if (bodies) *bodies = (int)W.bodies.size();
    if (fixtures) *fixtures = (int)W.fixtures.size();
    if (joints) *joints = (int)W.joints.size();
    if (contacts) {
        if (g->onDevice) {
            GB_CUDA(cudaStreamSynchronize(g->stream));
            WorldState st;
            GB_CUDA(cudaMemcpy(&st, g->batch.state + w, sizeof(WorldState), cudaMemcpyDeviceToHost));
            *contacts = st.contactCount;
        } else {
            *contacts = W.hasState ? W.state.contactCount : 0;
        }
    }
    return GB_OK;
}

gb_status gb_get_bodies(gb_world* g, int w, float* out)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || !out) return GB_ERR_INVALID;
    HWorld& W = g->worlds[w];
    const int nb = (int)W.bodies.size();
    if (g->onDevice) {
        GB_CUDA(cudaStreamSynchronize(g->stream));
        const WorldDesc& d = g->desc[w];
        std::vector<float4> xf(nb), sw(nb), sw0(nb), vel(nb);
        std::vector<int4> bi(nb);
        GB_CUDA(cudaMemcpy(xf.data(), g->batch.xf + d.bodyBase, nb * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(sw.data(), g->batch.sw + d.bodyBase, nb * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(sw0.data(), g->batch.sw0 + d.bodyBase, nb * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(vel.data(), g->batch.vel + d.bodyBase, nb * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(bi.data(), g->batch.bi + d.bodyBase, nb * sizeof(int4), cudaMemcpyDeviceToHost));
        for (int i = 0; i < nb; ++i) {
            float* o = out + 12 * i;
            o[0] = xf[i].x; o[1] = xf[i].y; o[2] = sw[i].z; o[3] = sw[i].x; o[4] = sw[i].y;
            o[5] = vel[i].x; o[6] = vel[i].y; o[7] = vel[i].z; o[8] = xf[i].z; o[9] = xf[i].w;
            o[10] = sw0[i].w; o[11] = (bi[i].y & kBAwake) ? 1.0f : 0.0f;
        }
    } else {
        for (int i = 0; i < nb; ++i) {
            const HBody& b = W.bodies[i];
            float* o = out + 12 * i;
            o[0] = b.xf.p.x; o[1] = b.xf.p.y; o[2] = b.sw.a; o[3] = b.sw.c.x; o[4] = b.sw.c.y;
            o[5] = b.v.x; o[6] = b.v.y; o[7] = b.w; o[8] = b.xf.q.s; o[9] = b.xf.q.c;
            o[10] = b.sleepTime; o[11] = (b.flags & kBAwake) ? 1.0f : 0.0f;
        }
    }
    return GB_OK;
}

gb_status gb_get_contacts(gb_world* g, int w, int* ints, float* floats, int cap, int* count)
{
    if (!g || w < 0 || w >= (int)g->worlds.size()) return GB_ERR_INVALID;
    HWorld& W = g->worlds[w];
    HContacts local;
    const HContacts* C = &W.contacts;
    int n = W.hasState ? W.state.contactCount : 0;
    if (g->onDevice) {
        GB_CUDA(cudaStreamSynchronize(g->stream));
        const WorldDesc& d = g->desc[w];
        WorldState st;
        GB_CUDA(cudaMemcpy(&st, g->batch.state + w, sizeof(WorldState), cudaMemcpyDeviceToHost));
        n = st.contactCount;
        int nc = d.contactCap;
        local.ci.resize(nc); local.mh.resize(nc); local.mv.resize(nc); local.mp0.resize(nc); local.mp1.resize(nc);
        local.order.resize(std::max(n, 1));
        GB_CUDA(cudaMemcpy(local.ci.data(), g->batch.ci + d.contactBase, nc * sizeof(int4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(local.mh.data(), g->batch.mh + d.contactBase, nc * sizeof(int4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(local.mv.data(), g->batch.mv + d.contactBase, nc * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(local.mp0.data(), g->batch.mp0 + d.contactBase, nc * sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(local.mp1.data(), g->batch.mp1 + d.contactBase, nc * sizeof(float4), cudaMemcpyDeviceToHost));
        if (n > 0)
            GB_CUDA(cudaMemcpy(local.order.data(), g->batch.order + 2 * (size_t)d.contactBase + st.orderStart,
                               n * sizeof(int), cudaMemcpyDeviceToHost));
        C = &local;
    }
    if (count) *count = n;
    for (int k = 0; k < n && k < cap; ++k) {
        int c = C->order[k];
        int4 info = C->ci[c], h = C->mh[c];
        float4 v = C->mv[c], p0 = C->mp0[c], p1 = C->mp1[c];
        bool any = h.y > 0;
        int* I = ints + 8 * k;
        float* F = floats + 12 * k;
        // fixture indices, the b2Contact flags, the toi counter; dead manifold fields zeroed
        I[0] = info.y; I[1] = info.z; I[2] = info.x; I[3] = h.y; I[4] = any ? h.x : 0;
        I[5] = h.y > 0 ? h.z : 0; I[6] = h.y > 1 ? h.w : 0;
        I[7] = info.w;
        F[0] = any ? v.x : 0.0f; F[1] = any ? v.y : 0.0f; F[2] = any ? v.z : 0.0f; F[3] = any ? v.w : 0.0f;
        F[4] = h.y > 0 ? p0.x : 0.0f; F[5] = h.y > 0 ? p0.y : 0.0f; F[6] = h.y > 0 ? p0.z : 0.0f; F[7] = h.y > 0 ? p0.w : 0.0f;
        F[8] = h.y > 1 ? p1.x : 0.0f; F[9] = h.y > 1 ? p1.y : 0.0f; F[10] = h.y > 1 ? p1.z : 0.0f; F[11] = h.y > 1 ? p1.w : 0.0f;
    }
    return GB_OK;
}

gb_status gb_get_proxies(gb_world* g, int w, int* proxy_ids, float* fat_aabbs)
{
    if (!g || w < 0 || w >= (int)g->worlds.size()) return GB_ERR_INVALID;
    HWorld& W = g->worlds[w];
    std::vector<float4> fat = W.fat;
    if (g->onDevice) {
        GB_CUDA(cudaStreamSynchronize(g->stream));
        const WorldDesc& d = g->desc[w];
        fat.resize(d.proxyCap);
        GB_CUDA(cudaMemcpy(fat.data(), g->batch.fat + d.proxyBase, d.proxyCap * sizeof(float4), cudaMemcpyDeviceToHost));
    }
    for (size_t i = 0; i < W.fixtures.size(); ++i) {
        int id = W.fixtures[i].proxyId;
        if (proxy_ids) proxy_ids[i] = id;
        if (fat_aabbs && id >= 0) {
            fat_aabbs[4 * i] = fat[id].x; fat_aabbs[4 * i + 1] = fat[id].y;
            fat_aabbs[4 * i + 2] = fat[id].z; fat_aabbs[4 * i + 3] = fat[id].w;
        }
    }
    return GB_OK;
}

gb_status gb_world_stats(gb_world* g, int w, int* islands, int* toi_events)
{
    if (!g || w < 0 || w >= (int)g->worlds.size()) return GB_ERR_INVALID;
    WorldState st = g->worlds[w].state;
    if (g->onDevice) {
        GB_CUDA(cudaStreamSynchronize(g->stream));
        GB_CUDA(cudaMemcpy(&st, g->batch.state + w, sizeof(WorldState), cudaMemcpyDeviceToHost));
    }
    if (islands) *islands = st.islands;
    if (toi_events) *toi_events = st.toiEvents;
    return GB_OK;
}

gb_status gb_world_totals(gb_world* g, long long* out)
{
    if (!g || !out) return GB_ERR_INVALID;
    for (int i = 0; i < 8; ++i) out[i] = 0;
    const int nw = (int)g->worlds.size();
    std::vector<WorldState> st(nw);
    if (g->onDevice) {
        GB_CUDA(cudaStreamSynchronize(g->stream));
        GB_CUDA(cudaMemcpy(st.data(), g->batch.state, nw * sizeof(WorldState), cudaMemcpyDeviceToHost));
    } else {
        for (int i = 0; i < nw; ++i) st[i] = g->worlds[i].state;
    }
    for (int i = 0; i < nw; ++i) {
        const HWorld& W = g->worlds[i];
        out[0] += st[i].contactCount;
        out[1] += st[i].solvedBodies;
        out[2] += st[i].solvedContacts;
        out[3] += st[i].pairsFound;
        out[4] += st[i].islands;
        out[5] += st[i].toiEvents;
        out[6] += W.proxyCount;
        for (const HBody& b : W.bodies) out[7] += b.type == kDynamic ? 1 : 0;
    }
    return GB_OK;
}

gb_status gb_world_profile(gb_world* g, unsigned long long* out)
{
    if (!g || !out) return GB_ERR_INVALID;
    const int nw = (int)g->worlds.size();
    std::vector<WorldState> st(nw);
    if (g->onDevice) {
        GB_CUDA(cudaStreamSynchronize(g->stream));
        GB_CUDA(cudaMemcpy(st.data(), g->batch.state, nw * sizeof(WorldState), cudaMemcpyDeviceToHost));
    } else {
        for (int i = 0; i < nw; ++i) st[i] = g->worlds[i].state;
    }
    for (int i = 0; i < nw; ++i)
        for (int k = 0; k < kProfileSlots; ++k) out[(size_t)kProfileSlots * i + k] = st[i].cyc[k];
    return GB_OK;
}

gb_status gb_world_stage_times(gb_world* g, float dt, int vi, int pi, float* ms)
{
    if (!g || !ms || vi < 0 || pi < 0 || g->tuneIndex >= 0) return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    cudaEvent_t e[5] = {};
    cudaError_t err = cudaSuccess;
    for (int i = 0; i < 5 && err == cudaSuccess; ++i) err = cudaEventCreate(&e[i]);
    const StepParams P = MakeParams(g, dt, vi, pi);
    if (err == cudaSuccess) err = cudaEventRecord(e[0], g->stream);
    const int nw = (int)g->schedule.size();
    if (err == cudaSuccess) err = b2gLaunchNarrowphase(g->batch, g->dNpChunks, g->npChunkStart[nw], g->stream);
    if (err == cudaSuccess) err = cudaEventRecord(e[1], g->stream);
    if (err == cudaSuccess) s = LaunchClasses(g, P, g->plan, b2gLaunchStep);
    if (err == cudaSuccess && s == GB_OK) err = cudaEventRecord(e[2], g->stream);
    if (err == cudaSuccess && s == GB_OK) err = b2gLaunchToi(g->batch, P, g->dToiChunks, g->toiChunkStart[nw], g->stream);
    if (err == cudaSuccess && s == GB_OK) err = cudaEventRecord(e[3], g->stream);
    if (err == cudaSuccess && s == GB_OK) s = LaunchClasses(g, P, g->plan, b2gLaunchStepToi);
    if (err == cudaSuccess && s == GB_OK) err = cudaEventRecord(e[4], g->stream);
    if (err == cudaSuccess && s == GB_OK) err = cudaEventSynchronize(e[4]);
    for (int i = 0; i < 4 && err == cudaSuccess && s == GB_OK; ++i) err = cudaEventElapsedTime(&ms[i], e[i], e[i + 1]);
    for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
    if (err != cudaSuccess) return GB_ERR_CUDA;
    return s;
}

// Bodies of consecutive worlds are consecutive rows of the body columns (one row of padding only
// for a world without bodies), so whole-batch transfers are single copies.
static bool BodyRowsContiguous(const gb_world* g)
{
    for (const WorldDesc& d : g->desc)
        if (d.bodyCount == 0) return false;
    return true;
}

gb_status gb_set_forces(gb_world* g, const float* forces)
{
    if (!g || !forces) return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    if (BodyRowsContiguous(g)) {
        size_t n = 0;
        for (const WorldDesc& d : g->desc) n += d.bodyCount;
        GB_CUDA(cudaMemcpyAsync(g->batch.frc, forces, n * sizeof(float4), cudaMemcpyHostToDevice, g->stream));
        return GB_OK;
    }
    size_t off = 0;
    for (const WorldDesc& d : g->desc) {
        if (d.bodyCount > 0)
            GB_CUDA(cudaMemcpyAsync(g->batch.frc + d.bodyBase, forces + 4 * off, d.bodyCount * sizeof(float4),
                                    cudaMemcpyHostToDevice, g->stream));
        off += d.bodyCount;
    }
    return GB_OK;
}

// The streams, staging buffers (one body column of float4 each) and events of the pipelined
// transfers, created on first use and again when the body count changed.
gb_status EnsureTransfers(gb_world* g, size_t n)
{
    if (g->upStream && g->stageBodies == n) return GB_OK;
    ReleaseTransferResources(g);
    GB_CUDA(cudaStreamCreateWithFlags(&g->upStream, cudaStreamNonBlocking));
    GB_CUDA(cudaStreamCreateWithFlags(&g->downStream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
        GB_CUDA(cudaMalloc(&g->forceStage[i], std::max<size_t>(n, 1) * sizeof(float4)));
        GB_CUDA(cudaMalloc(&g->xfStage[i], std::max<size_t>(n, 1) * sizeof(float4)));
        for (cudaEvent_t* e : {&g->upDone[i], &g->forceTaken[i], &g->xfReady[i], &g->downDone[i]})
            GB_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    g->stageBodies = n;
    g->upCount = g->downCount = 0;
    return GB_OK;
}

gb_status gb_set_forces_async(gb_world* g, const float* forces)
{
    if (!g || !forces) return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    if (!BodyRowsContiguous(g)) return gb_set_forces(g, forces);
    size_t n = 0;
    for (const WorldDesc& d : g->desc) n += d.bodyCount;
    if ((s = EnsureTransfers(g, n)) != GB_OK) return s;
    const int i = (int)(g->upCount++ & 1u);
    // the upload stream refills buffer i once the handle's stream has taken its previous contents
    if (g->upCount > 2) GB_CUDA(cudaStreamWaitEvent(g->upStream, g->forceTaken[i], 0));
    GB_CUDA(cudaMemcpyAsync(g->forceStage[i], forces, n * sizeof(float4), cudaMemcpyHostToDevice, g->upStream));
    GB_CUDA(cudaEventRecord(g->upDone[i], g->upStream));
    GB_CUDA(cudaStreamWaitEvent(g->stream, g->upDone[i], 0));
    GB_CUDA(cudaMemcpyAsync(g->batch.frc, g->forceStage[i], n * sizeof(float4), cudaMemcpyDeviceToDevice, g->stream));
    GB_CUDA(cudaEventRecord(g->forceTaken[i], g->stream));
    return GB_OK;
}

gb_status gb_get_transforms_async(gb_world* g, float* xf)
{
    if (!g || !xf) return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    if (!BodyRowsContiguous(g)) return gb_get_transforms(g, xf);
    size_t n = 0;
    for (const WorldDesc& d : g->desc) n += d.bodyCount;
    if ((s = EnsureTransfers(g, n)) != GB_OK) return s;
    const int i = (int)(g->downCount++ & 1u);
    // the handle's stream refills buffer i once the download stream has sent its previous contents
    if (g->downCount > 2) GB_CUDA(cudaStreamWaitEvent(g->stream, g->downDone[i], 0));
    GB_CUDA(cudaMemcpyAsync(g->xfStage[i], g->batch.xf, n * sizeof(float4), cudaMemcpyDeviceToDevice, g->stream));
    GB_CUDA(cudaEventRecord(g->xfReady[i], g->stream));
    GB_CUDA(cudaStreamWaitEvent(g->downStream, g->xfReady[i], 0));
    GB_CUDA(cudaMemcpyAsync(xf, g->xfStage[i], n * sizeof(float4), cudaMemcpyDeviceToHost, g->downStream));
    GB_CUDA(cudaEventRecord(g->downDone[i], g->downStream));
    return GB_OK;
}

gb_status gb_get_transforms(gb_world* g, float* xf)
{
    if (!g || !xf) return GB_ERR_INVALID;
    gb_status s = Upload(g);
    if (s != GB_OK) return s;
    size_t off = 0;
    if (BodyRowsContiguous(g)) {
        for (const WorldDesc& d : g->desc) off += d.bodyCount;
        GB_CUDA(cudaMemcpyAsync(xf, g->batch.xf, off * sizeof(float4), cudaMemcpyDeviceToHost, g->stream));
    } else {
        for (const WorldDesc& d : g->desc) {
            if (d.bodyCount > 0)
                GB_CUDA(cudaMemcpyAsync(xf + 4 * off, g->batch.xf + d.bodyBase, d.bodyCount * sizeof(float4),
                                        cudaMemcpyDeviceToHost, g->stream));
            off += d.bodyCount;
        }
    }
    GB_CUDA(cudaStreamSynchronize(g->stream));
    return GB_OK;
}

gb_status gb_sincos(const float* x, float* s, float* c, int n)
{
    if (n <= 0) return GB_OK;
    float *dx = nullptr, *ds = nullptr, *dc = nullptr;
    // every allocation is checked into e, so a failure part way frees what was allocated before it
    cudaError_t e = cudaMalloc(&dx, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&ds, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dc, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = b2gLaunchSinCos(dx, ds, dc, n, 0);
    if (e == cudaSuccess) e = cudaMemcpy(s, ds, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(c, dc, n * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dx); cudaFree(ds); cudaFree(dc);
    return cudaErr(e);
}

gb_status gb_collide(int n, const int* type_a, const float* shape_a, const int* n_a, const float* xf_a,
                     const int* type_b, const float* shape_b, const int* n_b, const float* xf_b,
                     int* out_ints, float* out_floats)
{
    if (n <= 0) return GB_OK;
    std::vector<Shape> sa(n), sb(n);
    std::vector<float4> xa(n), xb(n);
    for (int i = 0; i < n; ++i) {
        if (type_a[i] < 0 || type_a[i] > 3 || type_b[i] < 0 || type_b[i] > 3) return GB_ERR_INVALID;
        sa[i] = MakeShape(type_a[i], shape_a + 16 * i, n_a[i]);
        sb[i] = MakeShape(type_b[i], shape_b + 16 * i, n_b[i]);
        if (sa[i].type == kCircle && sb[i].type != kCircle) return GB_ERR_INVALID;
        if (sa[i].type == kPolygon && sb[i].type == kEdge) return GB_ERR_INVALID;
        if (sa[i].type == kEdge && sb[i].type == kEdge) return GB_ERR_INVALID;
        xa[i] = make_float4(xf_a[4 * i], xf_a[4 * i + 1], xf_a[4 * i + 2], xf_a[4 * i + 3]);
        xb[i] = make_float4(xf_b[4 * i], xf_b[4 * i + 1], xf_b[4 * i + 2], xf_b[4 * i + 3]);
    }
    Shape *dsa = nullptr, *dsb = nullptr;
    float4 *dxa = nullptr, *dxb = nullptr, *dof = nullptr;
    int4* doi = nullptr;
    // every allocation is checked into e, so a failure part way frees what was allocated before it
    cudaError_t e = cudaMalloc(&dsa, n * sizeof(Shape));
    if (e == cudaSuccess) e = cudaMalloc(&dsb, n * sizeof(Shape));
    if (e == cudaSuccess) e = cudaMalloc(&dxa, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&dxb, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&doi, n * sizeof(int4));
    if (e == cudaSuccess) e = cudaMalloc(&dof, 3 * n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemcpy(dsa, sa.data(), n * sizeof(Shape), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dsb, sb.data(), n * sizeof(Shape), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dxa, xa.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dxb, xb.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = b2gLaunchCollide(n, dsa, dxa, dsb, dxb, doi, dof, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out_ints, doi, n * sizeof(int4), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(out_floats, dof, 3 * n * sizeof(float4), cudaMemcpyDeviceToHost);
    cudaFree(dsa); cudaFree(dsb); cudaFree(dxa); cudaFree(dxb); cudaFree(doi); cudaFree(dof);
    return cudaErr(e);
}

} // extern "C"

namespace {

// b2Body::SynchronizeFixtures (Dynamics/b2Body.cpp:443-455) on the host copy: each proxy's swept box
// and, when it left the fat box, a new fat box (b2DynamicTree::MoveProxy, b2DynamicTree.cpp:133-177)
// with the proxy marked moved.
void SyncFixturesHost(HWorld& W, int bi)
{
    const HBody& b = W.bodies[bi];
    Xf xf1;
    xf1.q = RotOf(b.sw.a0);
    xf1.p = b.sw.c0 - Mul(xf1.q, b.sw.localCenter);
    for (int f = b.fixtureList; f != kNullIdx; f = W.fixtures[f].next) {
        HFixture& fx = W.fixtures[f];
        if (fx.proxyId == kNullIdx) continue;
        const float4 a = Combine(ComputeAABB(fx.shape, xf1), ComputeAABB(fx.shape, b.xf));
        fx.aabb = a;
        if (Contains(W.fat[fx.proxyId], a)) continue;
        const Vec2 disp = b.xf.p - xf1.p;
        float4 nb = make_float4(a.x - kAabbExtension, a.y - kAabbExtension, a.z + kAabbExtension, a.w + kAabbExtension);
        const Vec2 dd = kAabbMultiplier * disp;
        if (dd.x < 0.0f) nb.x += dd.x; else nb.z += dd.x;
        if (dd.y < 0.0f) nb.y += dd.y; else nb.w += dd.y;
        W.fat[fx.proxyId] = nb;
        W.moved[fx.proxyId] = 1;
        if (W.trackTree) W.tree.Move(fx.proxyId, nb);
    }
}

// b2Body property changes between steps on the host copy (prop: GB_BODY_*): SetType
// (Dynamics/b2Body.cpp:115-166), SetActive (:456-499), SetFixedRotation (:501-520), SetBullet,
// SetSleepingAllowed, SetLinearDamping, SetAngularDamping, SetGravityScale (b2Body.h:593-682), with
// the reference's order of effects; destroyed contacts report EndContact calls.
gb_status SetBodyPropertyHost(HWorld& W, int bi, int prop, const float* v, Calls& calls)
{
    HBody& b = W.bodies[bi];
    const bool flag = v[0] != 0.0f;
    auto destroyContacts = [&]() {
        if (W.hasState)
            for (int e = W.bodies[bi].contactList; e != kNullIdx;) {
                const int c = e >> 1;
                e = NextContactEdge(W, e);
                DestroyContactHost(W, c, calls);
            }
        W.bodies[bi].contactList = kNullIdx;
    };
    switch (prop) {
    case GB_BODY_TYPE: {
        const int type = (int)v[0];
        if (type < 0 || type > 2) return GB_ERR_INVALID;
        if (b.type == type) return GB_OK;
        b.type = type;
        ResetMassData(W, bi);
        if (type == kStatic) {
            W.bodies[bi].v = V(0.0f, 0.0f);
            W.bodies[bi].w = 0.0f;
            W.bodies[bi].sw.a0 = W.bodies[bi].sw.a;
            W.bodies[bi].sw.c0 = W.bodies[bi].sw.c;
            SyncFixturesHost(W, bi);
        }
        WakeHost(W.bodies[bi]);
        W.bodies[bi].force = V(0.0f, 0.0f);
        W.bodies[bi].torque = 0.0f;
        destroyContacts();
        // b2BroadPhase::TouchProxy: the proxies are queried again at the next pair finding
        for (int f = W.bodies[bi].fixtureList; f != kNullIdx; f = W.fixtures[f].next)
            if (W.fixtures[f].proxyId != kNullIdx) W.moved[W.fixtures[f].proxyId] = 1;
        return GB_OK;
    }
    case GB_BODY_ACTIVE: {
        const bool active = (b.flags & kBActive) != 0;
        if (flag == active) return GB_OK;
        if (flag) {
            b.flags |= kBActive;
            // b2Fixture::CreateProxies (Dynamics/b2Fixture.cpp:121-137) in the fixture list's order
            for (int f = b.fixtureList; f != kNullIdx; f = W.fixtures[f].next) {
                HFixture& fx = W.fixtures[f];
                fx.aabb = ComputeAABB(fx.shape, b.xf);
                const float4 fat = make_float4(fx.aabb.x - kAabbExtension, fx.aabb.y - kAabbExtension,
                                               fx.aabb.z + kAabbExtension, fx.aabb.w + kAabbExtension);
                fx.proxyId = AllocateProxy(W, fat, f);
            }
        } else {
            b.flags &= ~kBActive;
            for (int f = b.fixtureList; f != kNullIdx; f = W.fixtures[f].next) {
                HFixture& fx = W.fixtures[f];
                if (fx.proxyId != kNullIdx) FreeProxy(W, fx.proxyId);
                fx.proxyId = kNullIdx;
            }
            destroyContacts();
        }
        return GB_OK;
    }
    case GB_BODY_FIXED_ROTATION: {
        const bool fixed = (b.flags & kBFixedRot) != 0;
        if (fixed == flag) return GB_OK;
        if (flag) b.flags |= kBFixedRot;
        else b.flags &= ~kBFixedRot;
        b.w = 0.0f;
        ResetMassData(W, bi);
        return GB_OK;
    }
    case GB_BODY_BULLET:
        if (flag) b.flags |= kBBullet;
        else b.flags &= ~kBBullet;
        return GB_OK;
    case GB_BODY_SLEEPING_ALLOWED:
        if (flag) {
            b.flags |= kBAutoSleep;
        } else {
            b.flags &= ~kBAutoSleep;
            WakeHost(b);
        }
        return GB_OK;
    case GB_BODY_LINEAR_DAMPING: b.linDamp = v[0]; return GB_OK;
    case GB_BODY_ANGULAR_DAMPING: b.angDamp = v[0]; return GB_OK;
    case GB_BODY_GRAVITY_SCALE: b.gravScale = v[0]; return GB_OK;
    case GB_BODY_MASS_DATA: {
        // b2Body::SetMassData (Dynamics/b2Body.cpp:355-394): v = mass, center x, center y, inertia about
        // the body origin; dynamic bodies only; the center of mass moves and its velocity follows
        if (b.type != kDynamic) return GB_OK;
        b.invMass = 0.0f;
        b.I = 0.0f;
        b.invI = 0.0f;
        b.mass = v[0] <= 0.0f ? 1.0f : v[0];
        b.invMass = 1.0f / b.mass;
        const Vec2 center = V(v[1], v[2]);
        if (v[3] > 0.0f && (b.flags & kBFixedRot) == 0) {
            b.I = v[3] - b.mass * Dot(center, center);
            b.invI = 1.0f / b.I;
        }
        const Vec2 oldCenter = b.sw.c;
        b.sw.localCenter = center;
        b.sw.c = Mul(b.xf, center);
        b.sw.c0 = b.sw.c;
        b.v = b.v + Cross(b.w, b.sw.c - oldCenter);
        return GB_OK;
    }
    case GB_BODY_RESET_MASS_DATA: ResetMassData(W, bi); return GB_OK;
    default: return GB_ERR_INVALID;
    }
}

// ---- world checkpoints: a versioned record of everything a later step reads (the host copy after the
// device state was pulled back), each column a count and its raw records. Records are copied whole,
// so a checkpoint restores only into a build with the same record layouts, which the header's sizes
// check.
constexpr unsigned kCheckpointMagic = 0x57473242u;  // "B2GW"
constexpr unsigned kCheckpointVersion = 1;

template <typename T> void PutColumn(std::vector<unsigned char>& out, const std::vector<T>& v)
{
    static_assert(std::is_trivially_copyable<T>::value, "checkpoint columns are raw records");
    const long long n = (long long)v.size();
    const unsigned char* b = reinterpret_cast<const unsigned char*>(&n);
    out.insert(out.end(), b, b + sizeof(n));
    if (n > 0) {
        const unsigned char* d = reinterpret_cast<const unsigned char*>(v.data());
        out.insert(out.end(), d, d + n * sizeof(T));
    }
}
template <typename T> void PutValue(std::vector<unsigned char>& out, const T& x)
{
    static_assert(std::is_trivially_copyable<T>::value, "checkpoint values are raw records");
    const unsigned char* b = reinterpret_cast<const unsigned char*>(&x);
    out.insert(out.end(), b, b + sizeof(T));
}
template <typename T> bool GetColumn(const unsigned char*& p, const unsigned char* end, std::vector<T>& v)
{
    long long n = 0;
    if ((size_t)(end - p) < sizeof(n)) return false;
    std::memcpy(&n, p, sizeof(n));
    p += sizeof(n);
    if (n < 0 || (unsigned long long)n > (unsigned long long)(end - p) / sizeof(T)) return false;
    v.resize((size_t)n);
    if (n > 0) std::memcpy(v.data(), p, (size_t)n * sizeof(T));
    p += (size_t)n * sizeof(T);
    return true;
}
template <typename T> bool GetValue(const unsigned char*& p, const unsigned char* end, T& x)
{
    if ((size_t)(end - p) < sizeof(T)) return false;
    std::memcpy(&x, p, sizeof(T));
    p += sizeof(T);
    return true;
}

// the record sizes a checkpoint was written with (a build with other layouts refuses it)
std::vector<int> CheckpointLayout()
{
    return {(int)sizeof(gb_world_def), (int)sizeof(HBody), (int)sizeof(HFixture), (int)sizeof(Joint),
            (int)sizeof(WorldState), (int)sizeof(int4), (int)sizeof(float4)};
}

void SaveWorld(const HWorld& W, std::vector<unsigned char>& out)
{
    PutValue(out, kCheckpointMagic);
    PutValue(out, kCheckpointVersion);
    PutColumn(out, CheckpointLayout());
    PutValue(out, W.def);
    const int flags[10] = {W.autoClear ? 1 : 0, W.bodyList, W.jointList, W.nodeFresh, W.proxyCount,
                           W.treeLost ? 1 : 0, W.newFixture, W.hasState ? 1 : 0,
                           W.trackTree && !W.treeIncomplete ? 1 : 0, 0};
    PutValue(out, flags);
    PutColumn(out, W.bodies);
    PutColumn(out, W.fixtures);
    PutColumn(out, W.joints);
    PutColumn(out, W.fat);
    PutColumn(out, W.pfix);
    PutColumn(out, W.moved);
    PutColumn(out, W.nodeFree);
    PutValue(out, W.state);
    const HContacts& C = W.contacts;
    PutColumn(out, C.ci); PutColumn(out, C.ce); PutColumn(out, C.mh);
    PutColumn(out, C.cp); PutColumn(out, C.mv); PutColumn(out, C.mp0); PutColumn(out, C.mp1);
    PutColumn(out, C.order); PutColumn(out, C.cnext);
    if (flags[8]) W.tree.Save(out);
}

// A checkpoint into W (whole or not at all). The indices inside are checked against the columns'
// sizes so that no later step reads outside them.
bool LoadWorld(HWorld& W, const unsigned char* p, const unsigned char* end)
{
    unsigned magic = 0, version = 0;
    if (!GetValue(p, end, magic) || !GetValue(p, end, version)) return false;
    if (magic != kCheckpointMagic || version != kCheckpointVersion) return false;
    std::vector<int> layout;
    if (!GetColumn(p, end, layout) || layout != CheckpointLayout()) return false;
    HWorld N;
    int flags[10];
    if (!GetValue(p, end, N.def) || !GetValue(p, end, flags)) return false;
    HContacts& C = N.contacts;
    if (!GetColumn(p, end, N.bodies) || !GetColumn(p, end, N.fixtures) || !GetColumn(p, end, N.joints) ||
        !GetColumn(p, end, N.fat) || !GetColumn(p, end, N.pfix) || !GetColumn(p, end, N.moved) ||
        !GetColumn(p, end, N.nodeFree) || !GetValue(p, end, N.state) || !GetColumn(p, end, C.ci) ||
        !GetColumn(p, end, C.ce) || !GetColumn(p, end, C.mh) || !GetColumn(p, end, C.cp) ||
        !GetColumn(p, end, C.mv) || !GetColumn(p, end, C.mp0) || !GetColumn(p, end, C.mp1) ||
        !GetColumn(p, end, C.order) || !GetColumn(p, end, C.cnext))
        return false;
    const bool hasTree = flags[8] != 0;
    if (hasTree && !N.tree.Load(p, end)) return false;
    if (p != end) return false;
    N.autoClear = flags[0] != 0;
    N.bodyList = flags[1];
    N.jointList = flags[2];
    N.nodeFresh = flags[3];
    N.proxyCount = flags[4];
    N.treeLost = flags[5] != 0;
    N.newFixture = flags[6];
    N.hasState = flags[7] != 0;
    // index ranges: bodies, fixtures and joints refer to each other, proxies to fixtures
    const int nb = (int)N.bodies.size(), nf = (int)N.fixtures.size(), nj = (int)N.joints.size();
    const int np = (int)N.fat.size();
    auto inRange = [](int i, int n) { return i == kNullIdx || (i >= 0 && i < n); };
    if (!inRange(N.bodyList, nb) || !inRange(N.jointList, nj) || (int)N.pfix.size() != np ||
        (int)N.moved.size() != np || N.nodeFresh < 0)
        return false;
    for (const HBody& b : N.bodies)
        if (!inRange(b.fixtureList, nf) || !inRange(b.next, nb) || b.type < 0 || b.type > 2) return false;
    for (const HFixture& f : N.fixtures)
        if (!inRange(f.body, nb) || !inRange(f.next, nf) || !inRange(f.proxyId, np) || f.shape.count < 0 ||
            f.shape.count > kMaxPolyVerts)
            return false;
    for (const Joint& j : N.joints)
        if (j.bodyA != kNullIdx && (!inRange(j.bodyA, nb) || !inRange(j.bodyB, nb) || j.type < 0 ||
                                    j.type >= kJointTypes))
            return false;
    for (int x : N.pfix)
        if (!inRange(x, nf)) return false;
    // the free list of tree node ids (a corrupt id would size the proxy columns)
    if (N.nodeFresh > 2 * np + 2) return false;
    for (int x : N.nodeFree)
        if (x < -1 || x >= N.nodeFresh) return false;
    for (const HFixture& f : N.fixtures)
        if (f.shape.type < 0 || f.shape.type > 3) return false;
    // joint list links and edges (edge id = 2 x joint + side)
    for (const Joint& j : N.joints) {
        if (j.bodyA == kNullIdx) continue;
        if (!inRange(j.prev, nj) || !inRange(j.next, nj)) return false;
        for (int side = 0; side < 2; ++side)
            if (!inRange(j.ePrev[side], 2 * nj) || !inRange(j.eNext[side], 2 * nj)) return false;
        if (j.type == kJointGear && (!inRange(j.bodyC, nb) || !inRange(j.bodyD, nb))) return false;
    }
    for (const HBody& b : N.bodies)
        if (!inRange(b.jointList, 2 * nj)) return false;
    if (N.hasState) {
        const size_t nc = C.ci.size();
        if (C.ce.size() != nc || C.mh.size() != nc || C.cp.size() != nc || C.mv.size() != nc ||
            C.mp0.size() != nc || C.mp1.size() != nc || C.order.size() != nc || C.cnext.size() != nc ||
            N.state.contactCount < 0 || (size_t)N.state.contactCount > nc || nc > (1u << 28))
            return false;
        const int ncap = (int)nc;
        // contact slots, edges (2 x slot + side) and list: every index the step follows stays in range
        if (!inRange(N.state.freeContact, ncap)) return false;
        for (int c = 0; c < ncap; ++c) {
            if (!inRange(C.cnext[c], ncap)) return false;
            const int4 e = C.ce[c];
            if (!inRange(e.x, 2 * ncap) || !inRange(e.y, 2 * ncap) || !inRange(e.z, 2 * ncap) || !inRange(e.w, 2 * ncap))
                return false;
        }
        for (int k = 0; k < N.state.contactCount; ++k) {
            const int c = C.order[k];
            if (c < 0 || c >= ncap) return false;
            if (C.ci[c].y < 0 || C.ci[c].y >= nf || C.ci[c].z < 0 || C.ci[c].z >= nf) return false;
            // manifold type and point count
            if (C.mh[c].x < 0 || C.mh[c].x > 2 || C.mh[c].y < 0 || C.mh[c].y > 2) return false;
        }
        for (const HBody& b : N.bodies)
            if (!inRange(b.contactList, 2 * ncap)) return false;
    }
    N.trackTree = W.trackTree;
    N.treeIncomplete = W.trackTree && !hasTree;
    if (!N.trackTree) N.tree = ProxyTree();
    W = std::move(N);
    return true;
}

// b2Fixture changes between steps on the host copy (prop: GB_FIXTURE_*): SetFriction, SetRestitution,
// SetDensity (Dynamics/b2Fixture.h:300-340), SetSensor (b2Fixture.cpp:418-425: the body wakes on a
// change), SetFilterData with Refilter (b2Fixture.cpp:181-214: the fixture's contacts are flagged for
// filtering at the next collide phase and its proxies are queried again). A chain (its first child's
// index) is one b2Fixture and changes with all of its children.
gb_status SetFixturePropertyHost(HWorld& W, int f, int prop, const float* v)
{
    const int body = W.fixtures[f].body;
    int last = f;
    if (W.fixtures[f].shape.type == kEdge && W.fixtures[f].shape.chain == 1)
        while (last + 1 < (int)W.fixtures.size() && W.fixtures[last + 1].body == body &&
               W.fixtures[last + 1].shape.chain == 2)
            ++last;
    switch (prop) {
    case GB_FIXTURE_FRICTION:
        for (int k = f; k <= last; ++k) W.fixtures[k].friction = v[0];
        return GB_OK;
    case GB_FIXTURE_RESTITUTION:
        for (int k = f; k <= last; ++k) W.fixtures[k].restitution = v[0];
        return GB_OK;
    case GB_FIXTURE_DENSITY:
        if (!(v[0] >= 0.0f)) return GB_ERR_INVALID;  // b2Fixture::SetDensity asserts a valid density >= 0
        for (int k = f; k <= last; ++k) W.fixtures[k].density = v[0];
        return GB_OK;
    case GB_FIXTURE_SENSOR: {
        const int sensor = v[0] != 0.0f ? 1 : 0;
        if (sensor == W.fixtures[f].sensor) return GB_OK;
        WakeHost(W.bodies[body]);
        for (int k = f; k <= last; ++k) W.fixtures[k].sensor = sensor;
        return GB_OK;
    }
    case GB_FIXTURE_FILTER: {
        for (int k = f; k <= last; ++k) {
            W.fixtures[k].category = (int)v[0] & 0xFFFF;
            W.fixtures[k].mask = (int)v[1] & 0xFFFF;
            W.fixtures[k].group = (int16_t)(int)v[2];
        }
        if (W.hasState) {
            HContacts& C = W.contacts;
            for (int e = W.bodies[body].contactList; e != kNullIdx; e = NextContactEdge(W, e)) {
                int4& ci = C.ci[e >> 1];
                if ((ci.y >= f && ci.y <= last) || (ci.z >= f && ci.z <= last)) ci.x |= kCFilter;
            }
        }
        for (int k = f; k <= last; ++k)
            if (W.fixtures[k].proxyId != kNullIdx) W.moved[W.fixtures[k].proxyId] = 1;
        return GB_OK;
    }
    default: return GB_ERR_INVALID;
    }
}

// Joint changes between steps on the host copy (prop: GB_JOINT_*), with the reference's wakes and limit
// impulse resets: b2RevoluteJoint::EnableMotor, SetMotorSpeed, SetMaxMotorTorque, EnableLimit,
// SetLimits (Dynamics/Joints/b2RevoluteJoint.cpp:419-483), the prismatic joint's
// (b2PrismaticJoint.cpp:546-604; translations in lowerAngle/upperAngle, the motor force in
// maxMotorTorque) and the wheel joint's (b2WheelJoint.cpp:377-396) counterparts; the length, spring,
// force and offset setters of the distance, weld, wheel, rope, friction, motor, gear and mouse joints
// (their headers; b2MotorJoint.cpp:228-284). A property the joint's type does not have is invalid.
gb_status SetJointPropertyHost(HWorld& W, int ji, int prop, const float* v)
{
    Joint& j = W.joints[ji];
    const int t = j.type;
    const bool motorised = t == kJointRevolute || t == kJointPrismatic || t == kJointWheel;
    const bool limited = t == kJointRevolute || t == kJointPrismatic;
    const bool spring = t == kJointDistance || t == kJointWeld || t == kJointWheel || t == kJointMouse;
    auto wake = [&]() {
        WakeHost(W.bodies[j.bodyA]);
        WakeHost(W.bodies[j.bodyB]);
    };
    switch (prop) {
    case GB_JOINT_MOTOR_SPEED:
        if (!motorised) return GB_ERR_INVALID;
        wake();
        j.motorSpeed = v[0];
        return GB_OK;
    case GB_JOINT_MAX_MOTOR:
        if (!motorised) return GB_ERR_INVALID;
        wake();
        j.maxMotorTorque = v[0];
        return GB_OK;
    case GB_JOINT_ENABLE_MOTOR:
        if (!motorised) return GB_ERR_INVALID;
        wake();
        j.enableMotor = v[0] != 0.0f ? 1 : 0;
        return GB_OK;
    case GB_JOINT_ENABLE_LIMIT: {
        if (!limited) return GB_ERR_INVALID;
        const int flag = v[0] != 0.0f ? 1 : 0;
        if (flag != j.enableLimit) {
            wake();
            j.enableLimit = flag;
            j.impulse[2] = 0.0f;
        }
        return GB_OK;
    }
    case GB_JOINT_LIMITS:
        if (!limited || !(v[0] <= v[1])) return GB_ERR_INVALID;
        if (v[0] != j.lowerAngle || v[1] != j.upperAngle) {
            wake();
            j.impulse[2] = 0.0f;
            j.lowerAngle = v[0];
            j.upperAngle = v[1];
        }
        return GB_OK;
    case GB_JOINT_LENGTH:
        if (t != kJointDistance) return GB_ERR_INVALID;
        j.length = v[0];
        return GB_OK;
    case GB_JOINT_FREQUENCY:
        if (!spring) return GB_ERR_INVALID;
        j.frequencyHz = v[0];
        return GB_OK;
    case GB_JOINT_DAMPING_RATIO:
        if (!spring) return GB_ERR_INVALID;
        j.dampingRatio = v[0];
        return GB_OK;
    case GB_JOINT_MAX_LENGTH:
        if (t != kJointRope) return GB_ERR_INVALID;
        j.maxLength = v[0];
        return GB_OK;
    case GB_JOINT_MAX_FORCE:
        if (t != kJointFriction && t != kJointMotor && t != kJointMouse) return GB_ERR_INVALID;
        j.maxForce = v[0];
        return GB_OK;
    case GB_JOINT_MAX_TORQUE:
        if (t != kJointFriction && t != kJointMotor) return GB_ERR_INVALID;
        j.maxTorque = v[0];
        return GB_OK;
    case GB_JOINT_LINEAR_OFFSET:
        if (t != kJointMotor) return GB_ERR_INVALID;
        if (v[0] != j.linearOffset.x || v[1] != j.linearOffset.y) {
            wake();
            j.linearOffset = V(v[0], v[1]);
        }
        return GB_OK;
    case GB_JOINT_ANGULAR_OFFSET:
        if (t != kJointMotor) return GB_ERR_INVALID;
        if (v[0] != j.angularOffset) {
            wake();
            j.angularOffset = v[0];
        }
        return GB_OK;
    case GB_JOINT_CORRECTION_FACTOR:
        if (t != kJointMotor) return GB_ERR_INVALID;
        j.correctionFactor = v[0];
        return GB_OK;
    case GB_JOINT_RATIO:
        if (t != kJointGear) return GB_ERR_INVALID;
        j.ratio = v[0];
        return GB_OK;
    default: return GB_ERR_INVALID;
    }
}

} // namespace

extern "C" {

gb_status gb_polygon_shape(int mode, const float* in, int n, float* out, int* count)
{
    if (!in || !out || !count || mode < 0 || mode > 2 || (mode == 0 && (n < 0 || n > kMaxPolyVerts))) return GB_ERR_INVALID;
    Shape s;
    std::memset(&s, 0, sizeof(s));
    if (mode == 0) {
        Vec2 pts[kMaxPolyVerts];
        for (int i = 0; i < n; ++i) pts[i] = V(in[2 * i], in[2 * i + 1]);
        PolygonSet(s, pts, n);
    } else if (mode == 1) {
        PolygonSetAsBox(s, in[0], in[1]);
    } else {
        PolygonSetAsBox(s, in[0], in[1], V(in[2], in[3]), in[4]);
    }
    out[0] = s.centroid.x;
    out[1] = s.centroid.y;
    for (int i = 0; i < kMaxPolyVerts; ++i) {
        out[2 + 2 * i] = i < s.count ? s.v[i].x : 0.0f;
        out[3 + 2 * i] = i < s.count ? s.v[i].y : 0.0f;
        out[18 + 2 * i] = i < s.count ? s.n[i].x : 0.0f;
        out[19 + 2 * i] = i < s.count ? s.n[i].y : 0.0f;
    }
    *count = s.count;
    return GB_OK;
}

gb_status gb_fixture_query(gb_world* g, int w, int fixture, int op, const float* in, float* out)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || !out || (op < 2 && !in) || op < 0 || op > 3) return GB_ERR_INVALID;
    const HWorld& W = g->worlds[w];
    if (fixture < 0 || fixture >= (int)W.fixtures.size() || W.fixtures[fixture].body == kNullIdx) return GB_ERR_INVALID;
    const HFixture& fx = W.fixtures[fixture];
    const Shape& sh = fx.shape;
    Xf xf = W.bodies[fx.body].xf;
    float4 aabb = fx.aabb;
    if (g->onDevice) {
        // the body's transform and the proxy box of the last step live on the device
        const WorldDesc& d = g->desc[w];
        float4 x;
        GB_CUDA(cudaStreamSynchronize(g->stream));
        GB_CUDA(cudaMemcpy(&x, g->batch.xf + d.bodyBase + fx.body, sizeof(float4), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(&aabb, g->batch.faabb + d.fixBase + fixture, sizeof(float4), cudaMemcpyDeviceToHost));
        xf.p = V(x.x, x.y);
        xf.q.s = x.z;
        xf.q.c = x.w;
    }
    out[0] = out[1] = out[2] = out[3] = 0.0f;
    if (op == 0) {
        // b2Shape::TestPoint (Collision/Shapes/b2CircleShape.cpp:37-42, b2PolygonShape.cpp:255-268;
        // edges contain no point)
        const Vec2 p = V(in[0], in[1]);
        bool inside = false;
        if (sh.type == kCircle) {
            const Vec2 center = xf.p + Mul(xf.q, sh.v[0]);
            const Vec2 dd = p - center;
            inside = Dot(dd, dd) <= sh.radius * sh.radius;
        } else if (sh.type == kPolygon) {
            const Vec2 local = MulT(xf.q, p - xf.p);
            inside = true;
            for (int i = 0; i < sh.count && inside; ++i)
                if (Dot(sh.n[i], local - sh.v[i]) > 0.0f) inside = false;
        }
        out[0] = inside ? 1.0f : 0.0f;
    } else if (op == 1) {
        // b2Fixture::RayCast of the first child (b2Fixture.h:333-336)
        float fraction = 0.0f;
        Vec2 normal = V(0.0f, 0.0f);
        if (RayCastShape(sh, xf, V(in[0], in[1]), V(in[2], in[3]), in[4], &fraction, &normal)) {
            out[0] = 1.0f;
            out[1] = normal.x;
            out[2] = normal.y;
            out[3] = fraction;
        }
    } else if (op == 3) {
        // b2Fixture::GetMassData (b2Fixture.h:344-347): b2Shape::ComputeMass with the fixture's density
        MassData md;
        ComputeMass(sh, fx.density, &md);
        out[0] = md.mass;
        out[1] = md.center.x;
        out[2] = md.center.y;
        out[3] = md.I;
    } else {
        // b2Fixture::GetAABB (b2Fixture.h:338-342): the proxy's swept box of the last synchronisation
        out[0] = aabb.x;
        out[1] = aabb.y;
        out[2] = aabb.z;
        out[3] = aabb.w;
    }
    return GB_OK;
}

gb_status gb_get_joint_reaction(gb_world* g, int w, int joint, float inv_dt, float* out)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || !out) return GB_ERR_INVALID;
    const HWorld& W = g->worlds[w];
    if (joint < 0 || joint >= (int)W.joints.size() || W.joints[joint].bodyA == kNullIdx) return GB_ERR_INVALID;
    Joint j = W.joints[joint];
    if (g->onDevice) {
        // the impulses and axes of the last step live on the device
        GB_CUDA(cudaStreamSynchronize(g->stream));
        GB_CUDA(cudaMemcpy(&j, g->batch.joint + g->desc[w].jointBase + joint, sizeof(Joint), cudaMemcpyDeviceToHost));
    }
    // b2Joint::GetReactionForce, GetReactionTorque of each type (Dynamics/Joints/*.cpp), in the
    // reference's operation order
    Vec2 F = V(0.0f, 0.0f);
    float T = 0.0f;
    switch (j.type) {
    case kJointRevolute:
    case kJointWeld:
    case kJointFriction:
    case kJointMotor:
        F = V(inv_dt * j.impulse[0], inv_dt * j.impulse[1]);
        T = inv_dt * j.impulse[2];
        break;
    case kJointPrismatic: {
        const float k = j.motorImpulse + j.impulse[2];
        F = V(inv_dt * (j.impulse[0] * j.perp.x + k * j.u.x), inv_dt * (j.impulse[0] * j.perp.y + k * j.u.y));
        T = inv_dt * j.impulse[1];
        break;
    }
    case kJointDistance:
    case kJointRope: {
        const float s = inv_dt * j.impulse[0];
        F = V(s * j.u.x, s * j.u.y);
        break;
    }
    case kJointWheel:
        F = V(inv_dt * (j.impulse[0] * j.ay.x + j.springImpulse * j.ax.x),
              inv_dt * (j.impulse[0] * j.ay.y + j.springImpulse * j.ax.y));
        T = inv_dt * j.motorImpulse;
        break;
    case kJointMouse:
        F = V(inv_dt * j.impulse[0], inv_dt * j.impulse[1]);
        T = inv_dt * 0.0f;
        break;
    case kJointPulley:
        F = V(inv_dt * (j.impulse[0] * j.uB.x), inv_dt * (j.impulse[0] * j.uB.y));
        break;
    case kJointGear:
        F = V(inv_dt * (j.impulse[0] * j.JvAC.x), inv_dt * (j.impulse[0] * j.JvAC.y));
        T = inv_dt * (j.impulse[0] * j.JwA);
        break;
    default: break;
    }
    out[0] = F.x;
    out[1] = F.y;
    out[2] = T;
    return GB_OK;
}

gb_status gb_joint_set(gb_world* g, int w, int joint, int prop, const float* v)
{
    if (!v) return GB_ERR_INVALID;
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    HWorld& W = g->worlds[w];
    if (joint < 0 || joint >= (int)W.joints.size() || W.joints[joint].bodyA == kNullIdx) return GB_ERR_INVALID;
    return SetJointPropertyHost(W, joint, prop, v);
}

gb_status gb_world_shift_origin(gb_world* g, int w, float x, float y)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    HWorld& W = g->worlds[w];
    // b2World::ShiftOrigin (Dynamics/b2World.cpp:1261-1282)
    const Vec2 o = V(x, y);
    for (int b = W.bodyList; b != kNullIdx; b = W.bodies[b].next) {
        HBody& hb = W.bodies[b];
        hb.xf.p = hb.xf.p - o;
        hb.sw.c0 = hb.sw.c0 - o;
        hb.sw.c = hb.sw.c - o;
    }
    for (Joint& j : W.joints) {
        if (j.type == kJointMouse) j.target = j.target - o;  // b2MouseJoint::ShiftOrigin (b2MouseJoint.cpp:222)
        if (j.type == kJointPulley) {                        // b2PulleyJoint::ShiftOrigin (b2PulleyJoint.cpp:347)
            j.groundAnchorA = j.groundAnchorA - o;
            j.groundAnchorB = j.groundAnchorB - o;
        }
    }
    // b2BroadPhase::ShiftOrigin: the tree's boxes (the proxies' fat boxes; the fixtures' own boxes are
    // left as the reference leaves them)
    for (float4& f : W.fat) f = make_float4(f.x - x, f.y - y, f.z - x, f.w - y);
    if (W.trackTree) W.tree.ShiftOrigin(x, y);
    return GB_OK;
}

gb_status gb_fixture_set(gb_world* g, int w, int fixture, int prop, const float* v)
{
    if (!v) return GB_ERR_INVALID;
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    HWorld& W = g->worlds[w];
    if (fixture < 0 || fixture >= (int)W.fixtures.size() || W.fixtures[fixture].body == kNullIdx) return GB_ERR_INVALID;
    const Shape& sh = W.fixtures[fixture].shape;
    if (sh.type == kEdge && sh.chain == 2) return GB_ERR_INVALID;  // a chain goes by its first child
    return SetFixturePropertyHost(W, fixture, prop, v);
}

gb_status gb_world_checkpoint(gb_world* g, int w, void* buf, size_t cap, size_t* size)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || g->splitOpen || !size) return GB_ERR_INVALID;
    if (g->onDevice) {
        GB_CUDA(cudaStreamSynchronize(g->stream));
        if (g->upStream) GB_CUDA(cudaStreamSynchronize(g->upStream));
        if (g->downStream) GB_CUDA(cudaStreamSynchronize(g->downStream));
        // the world's device state as the host copy (the device keeps it: nothing is marked changed)
        gb_status s = Download(g);
        if (s != GB_OK) return s;
    }
    std::vector<unsigned char> out;
    SaveWorld(g->worlds[w], out);
    *size = out.size();
    if (!buf || cap < out.size()) return buf ? GB_ERR_CAPACITY : GB_OK;
    std::memcpy(buf, out.data(), out.size());
    return GB_OK;
}

gb_status gb_world_restore(gb_world* g, int w, const void* buf, size_t size)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || !buf || g->splitOpen || g->locked) return GB_ERR_INVALID;
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    const unsigned char* p = static_cast<const unsigned char*>(buf);
    if (!LoadWorld(g->worlds[w], p, p + size)) return GB_ERR_INVALID;
    ReleaseGraph(g);
    if (g->filterFn) {
        // verdicts of the world's old fixture pairs are decided again when met
        std::vector<unsigned long long> keys((size_t)g->filterCap);
        std::vector<int> vals((size_t)g->filterCap);
        GB_CUDA(cudaMemcpy(keys.data(), g->dFilterKeys, g->filterCap * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemcpy(vals.data(), g->dFilterVals, g->filterCap * sizeof(int), cudaMemcpyDeviceToHost));
        std::vector<unsigned long long> kk;
        std::vector<int> vv;
        for (int i = 0; i < g->filterCap; ++i)
            if (keys[i] != ~0ull && (int)(keys[i] >> 40) != w) {
                kk.push_back(keys[i]);
                vv.push_back(vals[i]);
            }
        s = BuildFilterTable(g, g->filterCap, kk, vv);
        if (s != GB_OK) return s;
        AttachFilter(g);
    }
    return GB_OK;
}

gb_status gb_world_track_tree(gb_world* g, int on)
{
    if (!g || g->splitOpen) return GB_ERR_INVALID;
    for (const HWorld& W : g->worlds)
        if (W.nodeFresh != 0) return GB_ERR_INVALID;  // a proxy exists or existed: its history is gone
    g->treeTrack = on != 0;
    for (HWorld& W : g->worlds) {
        W.trackTree = g->treeTrack;
        W.treeIncomplete = false;
        W.tree = ProxyTree();
    }
    ReleaseGraph(g);
    g->hostDirty = true;  // the next upload allocates (or drops) the device's tree log
    return GB_OK;
}

gb_status gb_world_tree_stats(gb_world* g, int w, int* height, int* balance, float* quality)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || !g->treeTrack || g->splitOpen) return GB_ERR_INVALID;
    if (g->onDevice) {
        GB_CUDA(cudaStreamSynchronize(g->stream));
        if (g->upStream) GB_CUDA(cudaStreamSynchronize(g->upStream));
        if (g->downStream) GB_CUDA(cudaStreamSynchronize(g->downStream));
        gb_status s = DrainTreeLog(g);
        if (s != GB_OK) return s;
    }
    const HWorld& W = g->worlds[w];
    if (W.treeIncomplete) return GB_ERR_CAPACITY;
    if (height) *height = W.tree.Height();
    if (balance) *balance = W.tree.MaxBalance();
    if (quality) *quality = W.tree.AreaRatio();
    return GB_OK;
}

gb_status gb_get_body_info(gb_world* g, int w, int body, float* out, int* flags)
{
    if (!g || w < 0 || w >= (int)g->worlds.size() || !out) return GB_ERR_INVALID;
    const HWorld& W = g->worlds[w];
    if (body < 0 || body >= (int)W.bodies.size() || !W.bodies[body].alive) return GB_ERR_INVALID;
    // mass data, damping and flags other than awake change only on the host, so its copy is current
    const HBody& b = W.bodies[body];
    out[0] = b.mass;
    out[1] = b.I + b.mass * Dot(b.sw.localCenter, b.sw.localCenter);  // b2Body::GetInertia (b2Body.h:546)
    out[2] = b.sw.localCenter.x;
    out[3] = b.sw.localCenter.y;
    out[4] = b.linDamp;
    out[5] = b.angDamp;
    out[6] = b.gravScale;
    if (flags)
        *flags = b.type | ((b.flags & kBBullet) ? 4 : 0) | ((b.flags & kBFixedRot) ? 8 : 0) |
                 ((b.flags & kBAutoSleep) ? 16 : 0) | ((b.flags & kBActive) ? 32 : 0);
    return GB_OK;
}

gb_status gb_body_set(gb_world* g, int w, int body, int prop, const float* v, int* calls, int cap, int* n_calls)
{
    if (!v) return GB_ERR_INVALID;
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    HWorld& W = g->worlds[w];
    if (body < 0 || body >= (int)W.bodies.size() || !W.bodies[body].alive) return GB_ERR_INVALID;
    Calls c;
    if ((s = SetBodyPropertyHost(W, body, prop, v, c)) != GB_OK) return s;
    return Finish(c, calls, cap, n_calls);
}

gb_status gb_destroy_body(gb_world* g, int w, int body, int* calls, int cap, int* n_calls)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    HWorld& W = g->worlds[w];
    if (body < 0 || body >= (int)W.bodies.size() || !W.bodies[body].alive) return GB_ERR_INVALID;
    Calls c;
    DestroyBodyHost(W, body, c);
    return Finish(c, calls, cap, n_calls);
}

gb_status gb_destroy_joint(gb_world* g, int w, int joint, int* calls, int cap, int* n_calls)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    HWorld& W = g->worlds[w];
    if (joint < 0 || joint >= (int)W.joints.size() || W.joints[joint].bodyA == kNullIdx) return GB_ERR_INVALID;
    Calls c;
    DestroyJointHost(W, joint);
    return Finish(c, calls, cap, n_calls);
}

gb_status gb_destroy_fixture(gb_world* g, int w, int fixture, int* calls, int cap, int* n_calls)
{
    gb_status s = Mutable(g, w);
    if (s != GB_OK) return s;
    HWorld& W = g->worlds[w];
    if (fixture < 0 || fixture >= (int)W.fixtures.size() || W.fixtures[fixture].body == kNullIdx) return GB_ERR_INVALID;
    const Shape& sh = W.fixtures[fixture].shape;
    if (sh.type == kEdge && sh.chain == 2) return GB_ERR_INVALID;  // a chain goes by its first child
    Calls c;
    DestroyFixtureHost(W, fixture, c);
    return Finish(c, calls, cap, n_calls);
}

const char* gb_version(void) { return "box2d_gb300 0.1 (Box2D 2.3.2 step semantics, sm_103a)"; }

} // extern "C"

// ------------------------------------------------------------------ narrowphase without allocation
// gb_collide_noalloc stages its inputs and outputs in one fixed device buffer defined here (static
// device storage for GB_COLLIDE_NOALLOC_MAX_PAIRS pairs) instead of allocating per call. The
// buffer's address is resolved once per device, with that device current, and cached; each call
// checks that the cached address is still device memory of the current context (a cudaDeviceReset
// moves the buffer) and resolves it again when it is not.
namespace {

constexpr int kNoAllocMaxDevices = 64;
constexpr size_t RoundUp256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kNaShapes = RoundUp256(sizeof(Shape) * GB_COLLIDE_NOALLOC_MAX_PAIRS);
constexpr size_t kNaXf = RoundUp256(sizeof(float4) * GB_COLLIDE_NOALLOC_MAX_PAIRS);
constexpr size_t kNaOi = RoundUp256(sizeof(int4) * GB_COLLIDE_NOALLOC_MAX_PAIRS);
constexpr size_t kNaOf = RoundUp256(3 * sizeof(float4) * GB_COLLIDE_NOALLOC_MAX_PAIRS);
constexpr size_t kNaBytes = 2 * kNaShapes + 2 * kNaXf + kNaOi + kNaOf;

} // namespace

static __device__ __align__(256) unsigned char gCollideScratch[kNaBytes];

namespace {

std::mutex gCollideScratchMutex;
unsigned char* gCollideScratchAddr[kNoAllocMaxDevices];

gb_status CollideScratch(unsigned char** out)
{
    int dev = -1;
    GB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return GB_ERR_INVALID;
    std::lock_guard<std::mutex> lock(gCollideScratchMutex);
    if (gCollideScratchAddr[dev] != nullptr) {
        // A cudaDeviceReset in this process ends the context the cached address belongs to; the
        // buffer then lives at a new address in the next context. An address that is no longer
        // device memory of the current context is dropped and resolved again.
        cudaPointerAttributes a{};
        const cudaError_t e = cudaPointerGetAttributes(&a, gCollideScratchAddr[dev]);
        if (e != cudaSuccess || a.type != cudaMemoryTypeDevice || a.device != dev) {
            (void)cudaGetLastError();
            gCollideScratchAddr[dev] = nullptr;
        }
    }
    if (gCollideScratchAddr[dev] == nullptr) {
        void* p = nullptr;
        GB_CUDA(cudaGetSymbolAddress(&p, gCollideScratch));
        gCollideScratchAddr[dev] = static_cast<unsigned char*>(p);
    }
    *out = gCollideScratchAddr[dev];
    return GB_OK;
}

} // namespace

extern "C" gb_status gb_collide_noalloc(int n, const int* type_a, const float* shape_a, const int* n_a,
                                        const float* xf_a, const int* type_b, const float* shape_b, const int* n_b,
                                        const float* xf_b, int* out_ints, float* out_floats)
{
    if (n <= 0) return GB_OK;
    if (n > GB_COLLIDE_NOALLOC_MAX_PAIRS) {
        std::fprintf(stderr, "box2d_gb300: gb_collide_noalloc: %d pairs exceed the fixed buffer of %d\n", n,
                     GB_COLLIDE_NOALLOC_MAX_PAIRS);
        return GB_ERR_CAPACITY;
    }
    if (!type_a || !shape_a || !n_a || !xf_a || !type_b || !shape_b || !n_b || !xf_b || !out_ints || !out_floats)
        return GB_ERR_INVALID;
    // the pair rules of gb_collide, checked before any device work
    for (int i = 0; i < n; ++i) {
        const int ta = type_a[i], tb = type_b[i];
        if (ta < 0 || ta > 3 || tb < 0 || tb > 3) return GB_ERR_INVALID;
        if (ta == 0 && tb != 0) return GB_ERR_INVALID;
        if (ta >= 2 && tb == 1) return GB_ERR_INVALID;
        if (ta == 1 && tb == 1) return GB_ERR_INVALID;
    }
    unsigned char* base = nullptr;
    gb_status s = CollideScratch(&base);
    if (s != GB_OK) return s;
    Shape* dsa = reinterpret_cast<Shape*>(base);
    Shape* dsb = reinterpret_cast<Shape*>(base + kNaShapes);
    float4* dxa = reinterpret_cast<float4*>(base + 2 * kNaShapes);
    float4* dxb = reinterpret_cast<float4*>(base + 2 * kNaShapes + kNaXf);
    int4* doi = reinterpret_cast<int4*>(base + 2 * kNaShapes + 2 * kNaXf);
    float4* dof = reinterpret_cast<float4*>(base + 2 * kNaShapes + 2 * kNaXf + kNaOi);
    // host-side shape setup in chunks on the stack; a synchronous copy from pageable memory returns
    // once the source has been consumed, so the chunk buffers are reused safely
    constexpr int kChunk = 64;
    Shape sa[kChunk], sb[kChunk];
    float4 xa[kChunk], xb[kChunk];
    for (int i0 = 0; i0 < n; i0 += kChunk) {
        const int m = std::min(kChunk, n - i0);
        for (int k = 0; k < m; ++k) {
            const int i = i0 + k;
            sa[k] = MakeShape(type_a[i], shape_a + 16 * i, n_a[i]);
            sb[k] = MakeShape(type_b[i], shape_b + 16 * i, n_b[i]);
            xa[k] = make_float4(xf_a[4 * i], xf_a[4 * i + 1], xf_a[4 * i + 2], xf_a[4 * i + 3]);
            xb[k] = make_float4(xf_b[4 * i], xf_b[4 * i + 1], xf_b[4 * i + 2], xf_b[4 * i + 3]);
        }
        GB_CUDA(cudaMemcpy(dsa + i0, sa, m * sizeof(Shape), cudaMemcpyHostToDevice));
        GB_CUDA(cudaMemcpy(dsb + i0, sb, m * sizeof(Shape), cudaMemcpyHostToDevice));
        GB_CUDA(cudaMemcpy(dxa + i0, xa, m * sizeof(float4), cudaMemcpyHostToDevice));
        GB_CUDA(cudaMemcpy(dxb + i0, xb, m * sizeof(float4), cudaMemcpyHostToDevice));
    }
    GB_CUDA(b2gLaunchCollide(n, dsa, dxa, dsb, dxb, doi, dof, 0));
    GB_CUDA(cudaMemcpy(out_ints, doi, n * sizeof(int4), cudaMemcpyDeviceToHost));
    GB_CUDA(cudaMemcpy(out_floats, dof, 3 * n * sizeof(float4), cudaMemcpyDeviceToHost));
    return GB_OK;
}
