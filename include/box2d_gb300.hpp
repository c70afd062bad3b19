// C++ mirror of the reference's host API (Box2D 2.3.2 b2World, b2Body, b2Fixture, b2Contact, shapes,
// b2RevoluteJointDef, b2ContactListener: Box2D/Dynamics/b2World.h:43-288, b2Body.h, b2Fixture.h,
// Contacts/b2Contact.h, b2WorldCallbacks.h) over the C-ABI of libbox2d_gb300.so, header only.
//
// The signatures and semantics a b2World user relies on are kept: a world owns its bodies, fixtures
// and joints (stable pointers until the world is destroyed), definitions are copied, Step(dt,
// velocityIterations, positionIterations) advances the world, and body state is read through the
// b2Body getters. Differences, all of them consequences of the state living on the GPU:
//  - a Step is queued on the device; the first getter after it waits for it and reads every body
//    once (the getters of that step are then host reads);
//  - the world settings (SetGravity, SetAllowSleeping, SetWarmStarting, SetContinuousPhysics,
//    SetSubStepping, SetAutoClearForces) and ClearForces act between steps, as in the reference, and
//    so do the body properties (SetType, SetActive, SetFixedRotation, SetBullet, SetSleepingAllowed,
//    SetLinearDamping, SetAngularDamping, SetGravityScale), with EndContact for the contacts SetType
//    and SetActive(false) destroy;
//  - DestroyBody, DestroyJoint and DestroyFixture run between steps with the reference's order of
//    effects; the destroyed objects stay allocated (their pointers stay valid, but dead) until the
//    world is destroyed, and the destruction listener and the contact listener's EndContact are
//    called during the Destroy call, as in the reference;
//  - QueryAABB and RayCast call their callbacks in fixture-creation order (the reference's order is
//    its broadphase tree's, which the device does not keep), with the reference's protocol: a
//    QueryAABB callback that returns false ends the query; a RayCast callback's return value ignores
//    the fixture (-1), ends the cast (0) or clips the ray (a fraction); the results of callbacks that
//    do not depend on the order (closest hit, all hits) are the reference's;
//  - b2Contact::GetWorldManifold and the b2Body frame getters (GetWorldPoint, GetLocalPoint, ...)
//    compute on the host: bit-exact with the reference when the caller is compiled without
//    floating-point contraction (-ffp-contract=off);
//  - b2ContactListener calls are recorded on the device during the step, in the reference's order.
//    With a listener set, Step runs in two halves (gb_world_step_begin / gb_world_step_end): the
//    collide phase's BeginContact, EndContact and PreSolve are made between them, and what PreSolve
//    changes (SetEnabled, SetFriction, SetRestitution, SetTangentSpeed) acts on the rest of the step;
//    PostSolve (with the solver's impulses) and the continuous phase's calls follow the step. The
//    continuous phase's own PreSolve calls (contacts with a static, kinematic or bullet body at a time
//    of impact) are notifications.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <memory>
#include <utility>
#include <vector>

#include "box2d_gb300.h"

namespace box2d {

struct b2Vec2 {
    float x = 0.0f, y = 0.0f;
    b2Vec2() = default;
    b2Vec2(float x_, float y_) : x(x_), y(y_) {}
    void Set(float x_, float y_) { x = x_; y = y_; }
    void SetZero() { x = 0.0f; y = 0.0f; }
};
struct b2Rot {
    float s = 0.0f, c = 1.0f;
    float GetAngle() const { return std::atan2(s, c); }
};
struct b2Transform {
    b2Vec2 p;
    b2Rot q;
};

enum b2BodyType { b2_staticBody = 0, b2_kinematicBody = 1, b2_dynamicBody = 2 };

// b2MassData (Box2D/Collision/Shapes/b2Shape.h:28-38): mass, centroid relative to the body origin,
// rotational inertia about the body origin
struct b2MassData {
    float mass = 0.0f;
    b2Vec2 center;
    float I = 0.0f;
};

struct b2BodyDef {
    b2BodyType type = b2_staticBody;
    b2Vec2 position;
    float angle = 0.0f;
    b2Vec2 linearVelocity;
    float angularVelocity = 0.0f;
    float linearDamping = 0.0f;
    float angularDamping = 0.0f;
    bool allowSleep = true;
    bool awake = true;
    bool fixedRotation = false;
    bool bullet = false;
    bool active = true;
    float gravityScale = 1.0f;
    void* userData = nullptr;
};

// ---------------------------------------------------------------- shapes (Collision/Shapes/*.h)
class b2Shape {
public:
    enum Type { e_circle = 0, e_edge = 1, e_polygon = 2, e_chain = 3 };
    virtual ~b2Shape() = default;
    Type GetType() const { return m_type; }
    // C-ABI encoding (gb_create_fixtures): type code, 16 floats, count
    virtual void Encode(int* type, float* shape, int* n) const = 0;
    Type m_type = e_circle;
    float m_radius = 0.0f;
};

class b2CircleShape : public b2Shape {
public:
    b2CircleShape() { m_type = e_circle; }
    void Encode(int* type, float* shape, int* n) const override
    {
        *type = 0; *n = 1;
        shape[0] = m_p.x; shape[1] = m_p.y; shape[2] = m_radius;
    }
    b2Vec2 m_p;
};

class b2EdgeShape : public b2Shape {
public:
    b2EdgeShape() { m_type = e_edge; m_radius = 0.01f; }  // b2_polygonRadius, as the reference
    void Set(const b2Vec2& v1, const b2Vec2& v2) { m_vertex1 = v1; m_vertex2 = v2; m_hasVertex0 = m_hasVertex3 = false; }
    void Encode(int* type, float* shape, int* n) const override
    {
        *type = 1; *n = 2;
        const float v[10] = {m_vertex1.x, m_vertex1.y, m_vertex2.x, m_vertex2.y, m_vertex0.x, m_vertex0.y,
                             m_vertex3.x, m_vertex3.y, m_hasVertex0 ? 1.0f : 0.0f, m_hasVertex3 ? 1.0f : 0.0f};
        for (int i = 0; i < 10; ++i) shape[i] = v[i];
    }
    b2Vec2 m_vertex1, m_vertex2, m_vertex0, m_vertex3;
    bool m_hasVertex0 = false, m_hasVertex3 = false;
};

// b2ChainShape (Box2D/Collision/Shapes/b2ChainShape.h:33-94): a free-form sequence of edges, open
// (CreateChain, optional ghost vertices before the first and after the last vertex) or closed
// (CreateLoop). b2Body::CreateFixture makes it through gb_create_chain, one device fixture per child.
class b2ChainShape : public b2Shape {
public:
    b2ChainShape() { m_type = e_chain; m_radius = 0.01f; }
    void CreateLoop(const b2Vec2* vertices, int count)
    {
        m_vertices.assign(vertices, vertices + count);
        m_loop = true;
        m_hasPrevVertex = m_hasNextVertex = false;
    }
    void CreateChain(const b2Vec2* vertices, int count)
    {
        m_vertices.assign(vertices, vertices + count);
        m_loop = false;
        m_hasPrevVertex = m_hasNextVertex = false;
    }
    void SetPrevVertex(const b2Vec2& v) { m_prevVertex = v; m_hasPrevVertex = true; }
    void SetNextVertex(const b2Vec2& v) { m_nextVertex = v; m_hasNextVertex = true; }
    int GetChildCount() const
    {
        const int n = (int)m_vertices.size();
        return m_loop ? n : (n > 0 ? n - 1 : 0);
    }
    // b2ChainShape::GetChildEdge (b2ChainShape.cpp:112-142): child index's edge with its ghost vertices
    void GetChildEdge(b2EdgeShape* edge, int index) const
    {
        const int n = (int)m_vertices.size();
        auto at = [&](int i) { return m_vertices[m_loop ? i % n : i]; };
        const int last = GetChildCount() - 1;
        edge->m_radius = m_radius;
        edge->m_vertex1 = at(index);
        edge->m_vertex2 = at(index + 1);
        if (index > 0) { edge->m_vertex0 = at(index - 1); edge->m_hasVertex0 = true; }
        else if (m_loop) { edge->m_vertex0 = m_vertices[n - 1]; edge->m_hasVertex0 = true; }
        else { edge->m_vertex0 = m_prevVertex; edge->m_hasVertex0 = m_hasPrevVertex; }
        if (index < last) { edge->m_vertex3 = at(index + 2); edge->m_hasVertex3 = true; }
        else if (m_loop) { edge->m_vertex3 = m_vertices[1]; edge->m_hasVertex3 = true; }
        else { edge->m_vertex3 = m_nextVertex; edge->m_hasVertex3 = m_hasNextVertex; }
    }
    // no single record: b2World::AddFixture passes the vertices to gb_create_chain
    void Encode(int* type, float* shape, int* n) const override { *type = -1; *n = 0; (void)shape; }

    std::vector<b2Vec2> m_vertices;
    b2Vec2 m_prevVertex, m_nextVertex;
    bool m_hasPrevVertex = false, m_hasNextVertex = false, m_loop = false;
};

class b2PolygonShape : public b2Shape {
public:
    b2PolygonShape() { m_type = e_polygon; m_radius = 0.01f; }  // b2_polygonRadius, as the reference
    // b2PolygonShape::Set: the hull is computed by the library exactly as the reference does
    void Set(const b2Vec2* points, int count)
    {
        m_mode = kPoints;
        m_inputCount = count < 8 ? count : 8;
        float in[16];
        for (int i = 0; i < m_inputCount; ++i) {
            m_points[i] = points[i];
            in[2 * i] = points[i].x;
            in[2 * i + 1] = points[i].y;
        }
        Fill(0, in, m_inputCount);
    }
    void SetAsBox(float hx, float hy)
    {
        m_mode = kBox; m_hx = hx; m_hy = hy; m_oriented = false;
        const float in[2] = {hx, hy};
        Fill(1, in, 0);
    }
    void SetAsBox(float hx, float hy, const b2Vec2& center, float angle)
    {
        m_mode = kBox; m_hx = hx; m_hy = hy; m_center = center; m_angle = angle; m_oriented = true;
        const float in[5] = {hx, hy, center.x, center.y, angle};
        Fill(2, in, 0);
    }
    int GetVertexCount() const { return m_count; }
    const b2Vec2& GetVertex(int index) const { return m_vertices[index]; }
    // the shape as the reference's b2PolygonShape holds it (b2PolygonShape.h:86-89), filled by Set and
    // SetAsBox through gb_polygon_shape
    b2Vec2 m_centroid;
    b2Vec2 m_vertices[8];
    b2Vec2 m_normals[8];
    int m_count = 0;
    void Encode(int* type, float* shape, int* n) const override
    {
        if (m_mode == kBox) {
            *type = 3;
            shape[0] = m_hx; shape[1] = m_hy;
            if (m_oriented) { shape[2] = m_center.x; shape[3] = m_center.y; shape[4] = m_angle; *n = 5; }
            else *n = 2;
        } else {
            *type = 2; *n = m_inputCount;
            for (int i = 0; i < m_inputCount; ++i) { shape[2 * i] = m_points[i].x; shape[2 * i + 1] = m_points[i].y; }
        }
    }

private:
    void Fill(int mode, const float* in, int n)
    {
        float out[34] = {0};
        int count = 0;
        if (gb_polygon_shape(mode, in, n, out, &count) != GB_OK) return;
        m_centroid = b2Vec2(out[0], out[1]);
        m_count = count;
        for (int i = 0; i < 8; ++i) {
            m_vertices[i] = b2Vec2(out[2 + 2 * i], out[3 + 2 * i]);
            m_normals[i] = b2Vec2(out[18 + 2 * i], out[19 + 2 * i]);
        }
    }
    enum Mode { kPoints, kBox } m_mode = kBox;
    b2Vec2 m_points[8];
    int m_inputCount = 0;
    float m_hx = 0.0f, m_hy = 0.0f, m_angle = 0.0f;
    b2Vec2 m_center;
    bool m_oriented = false;
};

struct b2Filter {
    uint16_t categoryBits = 0x0001;
    uint16_t maskBits = 0xFFFF;
    int16_t groupIndex = 0;
};

struct b2FixtureDef {
    const b2Shape* shape = nullptr;
    void* userData = nullptr;
    float friction = 0.2f;
    float restitution = 0.0f;
    float density = 0.0f;
    bool isSensor = false;
    b2Filter filter;
};

class b2World;
class b2Body;
class b2Joint;

// b2AABB (Box2D/Collision/b2Collision.h:206-247)
struct b2AABB {
    b2Vec2 lowerBound, upperBound;
};
// b2RayCastInput, b2RayCastOutput (Box2D/Collision/b2Collision.h:153-166)
struct b2RayCastInput {
    b2Vec2 p1, p2;
    float maxFraction = 1.0f;
};
struct b2RayCastOutput {
    b2Vec2 normal;
    float fraction = 0.0f;
};

class b2Fixture {
public:
    b2Body* GetBody() const { return m_body; }
    int GetIndex() const { return m_index; }
    float GetFriction() const { return m_def.friction; }
    float GetRestitution() const { return m_def.restitution; }
    float GetDensity() const { return m_def.density; }
    bool IsSensor() const { return m_def.isSensor; }
    void* GetUserData() const { return m_def.userData; }
    void SetUserData(void* data) { m_def.userData = data; }
    // the next fixture of the body's list (newest first), as b2Fixture::GetNext
    b2Fixture* GetNext() const;
    b2Shape::Type GetType() const { return m_type; }
    float GetRadius() const { return m_radius; }  // the shape's m_radius
    const b2Filter& GetFilterData() const { return m_def.filter; }
    // changes between steps (Box2D/Dynamics/b2Fixture.h:300-340, b2Fixture.cpp:181-214, 418-425), each a
    // gb_fixture_set call: friction and restitution reach new contacts, density the next mass reset,
    // a sensor change wakes the body, new filter data filters the fixture's contacts again
    void SetFriction(float friction);
    void SetRestitution(float restitution);
    void SetDensity(float density);
    void SetSensor(bool sensor);
    void SetFilterData(const b2Filter& filter);
    void Refilter() { SetFilterData(m_def.filter); }
    // b2Fixture::TestPoint, RayCast, GetAABB (Box2D/Dynamics/b2Fixture.h:313-342) at the body's
    // current transform (gb_fixture_query); a chain's child by childIndex
    bool TestPoint(const b2Vec2& p) const;
    bool RayCast(b2RayCastOutput* output, const b2RayCastInput& input, int childIndex) const;
    const b2AABB GetAABB(int childIndex) const;
    void GetMassData(b2MassData* massData) const;

private:
    friend class b2World;
    friend class b2Body;
    b2Body* m_body = nullptr;
    int m_index = -1;
    size_t m_slot = 0;  // position in the world's fixtures (creation order)
    b2FixtureDef m_def;
    b2Shape::Type m_type = b2Shape::e_circle;
    float m_radius = 0.0f;
    bool m_alive = true;
};

class b2Contact;
// b2ContactEdge, b2JointEdge (Box2D/Dynamics/Contacts/b2Contact.h:70-76, Joints/b2Joint.h:63-69)
struct b2ContactEdge {
    b2Body* other = nullptr;
    b2Contact* contact = nullptr;
    b2ContactEdge* prev = nullptr;
    b2ContactEdge* next = nullptr;
};
struct b2JointEdge {
    b2Body* other = nullptr;
    b2Joint* joint = nullptr;
    b2JointEdge* prev = nullptr;
    b2JointEdge* next = nullptr;
};

class b2Body {
public:
    b2Fixture* CreateFixture(const b2FixtureDef* def);
    b2Fixture* CreateFixture(const b2Shape* shape, float density)
    {
        b2FixtureDef d;
        d.shape = shape;
        d.density = density;
        return CreateFixture(&d);
    }
    // b2Body::DestroyFixture (Box2D/Dynamics/b2Body.cpp:216-281)
    void DestroyFixture(b2Fixture* fixture);
    // the next body of the world's body list (newest first), as b2Body::GetNext
    b2Body* GetNext() const;
    b2BodyType GetType() const { return m_type; }
    int GetIndex() const { return m_index; }
    b2World* GetWorld() const { return m_world; }
    void* GetUserData() const { return m_userData; }
    void SetUserData(void* data) { m_userData = data; }
    // the body's fixture list (newest first), as b2Body::GetFixtureList
    b2Fixture* GetFixtureList() const;
    // the body's contact and joint edges (newest first, as the reference's lists), rebuilt at each
    // call from the world's contact list and joints: valid until the next call or step
    b2ContactEdge* GetContactList();
    b2JointEdge* GetJointList();
    const b2Vec2 GetPosition() const { const float* s = State(); return b2Vec2(s[0], s[1]); }
    float GetAngle() const { return State()[2]; }
    const b2Vec2 GetWorldCenter() const { const float* s = State(); return b2Vec2(s[3], s[4]); }
    const b2Vec2 GetLinearVelocity() const { const float* s = State(); return b2Vec2(s[5], s[6]); }
    float GetAngularVelocity() const { return State()[7]; }
    const b2Transform GetTransform() const
    {
        const float* s = State();
        b2Transform t;
        t.p = b2Vec2(s[0], s[1]);
        t.q.s = s[8];
        t.q.c = s[9];
        return t;
    }
    bool IsAwake() const { return State()[11] != 0.0f; }
    // frames (Box2D/Dynamics/b2Body.h:558-600), with the reference's operation order: b2Mul, b2MulT,
    // b2Cross of the body's transform, center and velocities
    b2Vec2 GetWorldPoint(const b2Vec2& local) const
    {
        const b2Transform t = GetTransform();
        return b2Vec2((t.q.c * local.x - t.q.s * local.y) + t.p.x, (t.q.s * local.x + t.q.c * local.y) + t.p.y);
    }
    b2Vec2 GetWorldVector(const b2Vec2& local) const
    {
        const b2Transform t = GetTransform();
        return b2Vec2(t.q.c * local.x - t.q.s * local.y, t.q.s * local.x + t.q.c * local.y);
    }
    b2Vec2 GetLocalPoint(const b2Vec2& world) const
    {
        const b2Transform t = GetTransform();
        const float px = world.x - t.p.x, py = world.y - t.p.y;
        return b2Vec2(t.q.c * px + t.q.s * py, -t.q.s * px + t.q.c * py);
    }
    b2Vec2 GetLocalVector(const b2Vec2& world) const
    {
        const b2Transform t = GetTransform();
        return b2Vec2(t.q.c * world.x + t.q.s * world.y, -t.q.s * world.x + t.q.c * world.y);
    }
    b2Vec2 GetLinearVelocityFromWorldPoint(const b2Vec2& world) const
    {
        const b2Vec2 v = GetLinearVelocity(), c = GetWorldCenter();
        const float w = GetAngularVelocity();
        return b2Vec2(v.x + -w * (world.y - c.y), v.y + w * (world.x - c.x));
    }
    b2Vec2 GetLinearVelocityFromLocalPoint(const b2Vec2& local) const
    {
        return GetLinearVelocityFromWorldPoint(GetWorldPoint(local));
    }
    // mass data, damping and flags (Box2D/Dynamics/b2Body.h:227-260, 546-556, 593-682), read from the
    // library's host copy (gb_get_body_info)
    float GetMass() const { return Info(0); }
    float GetInertia() const { return Info(1); }
    const b2Vec2 GetLocalCenter() const { return b2Vec2(Info(2), Info(3)); }
    void GetMassData(b2MassData* data) const
    {
        data->mass = Info(0);
        data->I = Info(1);
        data->center = b2Vec2(Info(2), Info(3));
    }
    float GetLinearDamping() const { return Info(4); }
    float GetAngularDamping() const { return Info(5); }
    float GetGravityScale() const { return Info(6); }
    bool IsBullet() const { return (InfoFlags() & 4) != 0; }
    bool IsFixedRotation() const { return (InfoFlags() & 8) != 0; }
    bool IsSleepingAllowed() const { return (InfoFlags() & 16) != 0; }
    bool IsActive() const { return (InfoFlags() & 32) != 0; }
    // State changes between steps (Box2D/Dynamics/b2Body.cpp:419, b2Body.h:501-830), each one
    // gb_body_edits record applied on the device in call order before the next Step, with the
    // reference's semantics (type checks, wakes, no accumulation on sleeping bodies).
    void SetTransform(const b2Vec2& position, float angle);
    void SetLinearVelocity(const b2Vec2& v);
    void SetAngularVelocity(float omega);
    void SetAwake(bool flag);
    void ApplyForce(const b2Vec2& force, const b2Vec2& point, bool wake);
    void ApplyForceToCenter(const b2Vec2& force, bool wake);
    void ApplyTorque(float torque, bool wake);
    void ApplyLinearImpulse(const b2Vec2& impulse, const b2Vec2& point, bool wake);
    void ApplyAngularImpulse(float impulse, bool wake);
    // Property changes between steps (Box2D/Dynamics/b2Body.cpp:115-166 SetType, :456-499
    // SetActive, :501-520 SetFixedRotation; b2Body.h:593-682), each one gb_body_set call; the
    // contacts SetType and SetActive(false) destroy make their EndContact calls.
    void SetType(b2BodyType type);
    void SetActive(bool flag);
    void SetFixedRotation(bool flag);
    void SetBullet(bool flag);
    void SetSleepingAllowed(bool flag);
    void SetLinearDamping(float linearDamping);
    void SetAngularDamping(float angularDamping);
    void SetGravityScale(float scale);
    // b2Body::SetMassData (Box2D/Dynamics/b2Body.cpp:355-394), ResetMassData (:283-353)
    void SetMassData(const b2MassData* data);
    void ResetMassData();

private:
    friend class b2World;
    const float* State() const;
    float Info(int k) const;
    int InfoFlags() const;
    b2World* m_world = nullptr;
    int m_index = -1;
    b2BodyType m_type = b2_staticBody;
    void* m_userData = nullptr;
    bool m_alive = true;
    std::vector<b2ContactEdge> m_contactEdges;
    std::vector<b2JointEdge> m_jointEdges;
};

struct b2RevoluteJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Vec2 localAnchorA, localAnchorB;
    float referenceAngle = 0.0f;
    bool enableLimit = false;
    float lowerAngle = 0.0f, upperAngle = 0.0f;
    bool enableMotor = false;
    float motorSpeed = 0.0f, maxMotorTorque = 0.0f;
    // b2RevoluteJointDef::Initialize (b2RevoluteJoint.cpp:40-47): anchor in world coordinates
    void Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor);
};

struct b2DistanceJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Vec2 localAnchorA, localAnchorB;
    float length = 1.0f;
    float frequencyHz = 0.0f, dampingRatio = 0.0f;
    // b2DistanceJointDef::Initialize (b2DistanceJoint.cpp:41-50): anchors in world coordinates
    void Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchorA, const b2Vec2& anchorB);
};

struct b2WeldJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Vec2 localAnchorA, localAnchorB;
    float referenceAngle = 0.0f;
    float frequencyHz = 0.0f, dampingRatio = 0.0f;
    // b2WeldJointDef::Initialize (b2WeldJoint.cpp:36-43)
    void Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor);
};

// b2WheelJointDef, b2RopeJointDef, b2FrictionJointDef, b2MotorJointDef (Box2D/Dynamics/Joints/
// b2WheelJoint.h:30-68, b2RopeJoint.h:28-45, b2FrictionJoint.h:25-45, b2MotorJoint.h:26-55), with
// the reference's defaults
struct b2WheelJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Vec2 localAnchorA, localAnchorB;
    b2Vec2 localAxisA{1.0f, 0.0f};
    bool enableMotor = false;
    float maxMotorTorque = 0.0f, motorSpeed = 0.0f;
    float frequencyHz = 2.0f, dampingRatio = 0.7f;
    // b2WheelJointDef::Initialize (b2WheelJoint.cpp:39-46)
    void Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor, const b2Vec2& axis);
};
struct b2RopeJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Vec2 localAnchorA{-1.0f, 0.0f}, localAnchorB{1.0f, 0.0f};
    float maxLength = 0.0f;
};
struct b2FrictionJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Vec2 localAnchorA, localAnchorB;
    float maxForce = 0.0f, maxTorque = 0.0f;
    // b2FrictionJointDef::Initialize (b2FrictionJoint.cpp:35-41)
    void Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor);
};
struct b2MotorJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Vec2 linearOffset;
    float angularOffset = 0.0f;
    float maxForce = 1.0f, maxTorque = 1.0f, correctionFactor = 0.3f;
    // b2MotorJointDef::Initialize (b2MotorJoint.cpp:35-44)
    void Initialize(b2Body* bA, b2Body* bB);
};

// b2MouseJointDef (Box2D/Dynamics/Joints/b2MouseJoint.h:28-56): body B's point under `target` is
// pulled to the target, which b2MouseJoint::SetTarget moves between steps
struct b2MouseJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Vec2 target;
    float maxForce = 0.0f, frequencyHz = 5.0f, dampingRatio = 0.7f;
};

// b2PulleyJointDef (Box2D/Dynamics/Joints/b2PulleyJoint.h:30-72): lengthA + ratio * lengthB constant
struct b2PulleyJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = true;
    b2Vec2 groundAnchorA{-1.0f, 1.0f}, groundAnchorB{1.0f, 1.0f};
    b2Vec2 localAnchorA{-1.0f, 0.0f}, localAnchorB{1.0f, 0.0f};
    float lengthA = 0.0f, lengthB = 0.0f, ratio = 1.0f;
    // b2PulleyJointDef::Initialize (b2PulleyJoint.cpp:37-51): anchors given in world coordinates
    void Initialize(b2Body* bA, b2Body* bB, const b2Vec2& groundA, const b2Vec2& groundB, const b2Vec2& anchorA,
                    const b2Vec2& anchorB, float r);
};

// b2GearJointDef (Box2D/Dynamics/Joints/b2GearJoint.h:26-46): joint1 and joint2 are revolute or
// prismatic joints created before it
class b2Joint;
struct b2GearJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Joint* joint1 = nullptr;
    b2Joint* joint2 = nullptr;
    float ratio = 1.0f;
};

// b2PrismaticJointDef (Box2D/Dynamics/Joints/b2PrismaticJoint.h:30-88)
struct b2PrismaticJointDef {
    void* userData = nullptr;
    b2Body* bodyA = nullptr;
    b2Body* bodyB = nullptr;
    bool collideConnected = false;
    b2Vec2 localAnchorA, localAnchorB;
    b2Vec2 localAxisA{1.0f, 0.0f};
    float referenceAngle = 0.0f;
    bool enableLimit = false;
    float lowerTranslation = 0.0f, upperTranslation = 0.0f;
    bool enableMotor = false;
    float maxMotorForce = 0.0f, motorSpeed = 0.0f;
    // b2PrismaticJointDef::Initialize (b2PrismaticJoint.cpp:92-100)
    void Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor, const b2Vec2& axis);
};

class b2Joint {
public:
    virtual ~b2Joint() = default;
    int GetIndex() const { return m_index; }
    b2Body* GetBodyA() const { return m_a; }
    b2Body* GetBodyB() const { return m_b; }
    void* GetUserData() const { return m_userData; }
    void SetUserData(void* data) { m_userData = data; }
    // the next joint of the world's joint list (newest first), as b2Joint::GetNext
    b2Joint* GetNext() const;
    // b2Joint::GetReactionForce / GetReactionTorque (Box2D/Dynamics/Joints/*.cpp) after the last step
    b2Vec2 GetReactionForce(float inv_dt) const;
    float GetReactionTorque(float inv_dt) const;

protected:
    friend class b2World;
    // one gb_joint_set call (GB_JOINT_*); false when it did not apply
    bool Set(int prop, float v0, float v1 = 0.0f);
    int m_index = -1;
    size_t m_slot = 0;  // position in the world's joints (creation order)
    b2Body *m_a = nullptr, *m_b = nullptr;
    b2World* m_world = nullptr;
    void* m_userData = nullptr;
    bool m_alive = true;
};

// The typed joints CreateJoint returns, so that the reference's static_cast<b2RevoluteJoint*> and its
// setters read the same (Box2D/Dynamics/Joints/*.h). Each setter is a gb_joint_set call with the
// reference's wakes and limit-impulse resets; the getters return what was defined or set.
class b2RevoluteJoint : public b2Joint {
public:
    void EnableMotor(bool flag) { if (Set(GB_JOINT_ENABLE_MOTOR, flag ? 1.0f : 0.0f)) m_enableMotor = flag; }
    void SetMotorSpeed(float speed) { if (Set(GB_JOINT_MOTOR_SPEED, speed)) m_motorSpeed = speed; }
    void SetMaxMotorTorque(float torque) { if (Set(GB_JOINT_MAX_MOTOR, torque)) m_maxMotorTorque = torque; }
    void EnableLimit(bool flag) { if (Set(GB_JOINT_ENABLE_LIMIT, flag ? 1.0f : 0.0f)) m_enableLimit = flag; }
    void SetLimits(float lower, float upper)
    {
        if (Set(GB_JOINT_LIMITS, lower, upper)) { m_lower = lower; m_upper = upper; }
    }
    bool IsMotorEnabled() const { return m_enableMotor; }
    float GetMotorSpeed() const { return m_motorSpeed; }
    float GetMaxMotorTorque() const { return m_maxMotorTorque; }
    bool IsLimitEnabled() const { return m_enableLimit; }
    float GetLowerLimit() const { return m_lower; }
    float GetUpperLimit() const { return m_upper; }

private:
    friend class b2World;
    bool m_enableMotor = false, m_enableLimit = false;
    float m_motorSpeed = 0.0f, m_maxMotorTorque = 0.0f, m_lower = 0.0f, m_upper = 0.0f;
};
class b2PrismaticJoint : public b2Joint {
public:
    void EnableMotor(bool flag) { if (Set(GB_JOINT_ENABLE_MOTOR, flag ? 1.0f : 0.0f)) m_enableMotor = flag; }
    void SetMotorSpeed(float speed) { if (Set(GB_JOINT_MOTOR_SPEED, speed)) m_motorSpeed = speed; }
    void SetMaxMotorForce(float force) { if (Set(GB_JOINT_MAX_MOTOR, force)) m_maxMotorForce = force; }
    void EnableLimit(bool flag) { if (Set(GB_JOINT_ENABLE_LIMIT, flag ? 1.0f : 0.0f)) m_enableLimit = flag; }
    void SetLimits(float lower, float upper)
    {
        if (Set(GB_JOINT_LIMITS, lower, upper)) { m_lower = lower; m_upper = upper; }
    }
    bool IsMotorEnabled() const { return m_enableMotor; }
    float GetMotorSpeed() const { return m_motorSpeed; }
    float GetMaxMotorForce() const { return m_maxMotorForce; }
    bool IsLimitEnabled() const { return m_enableLimit; }
    float GetLowerLimit() const { return m_lower; }
    float GetUpperLimit() const { return m_upper; }

private:
    friend class b2World;
    bool m_enableMotor = false, m_enableLimit = false;
    float m_motorSpeed = 0.0f, m_maxMotorForce = 0.0f, m_lower = 0.0f, m_upper = 0.0f;
};
class b2WheelJoint : public b2Joint {
public:
    void EnableMotor(bool flag) { if (Set(GB_JOINT_ENABLE_MOTOR, flag ? 1.0f : 0.0f)) m_enableMotor = flag; }
    void SetMotorSpeed(float speed) { if (Set(GB_JOINT_MOTOR_SPEED, speed)) m_motorSpeed = speed; }
    void SetMaxMotorTorque(float torque) { if (Set(GB_JOINT_MAX_MOTOR, torque)) m_maxMotorTorque = torque; }
    void SetSpringFrequencyHz(float hz) { if (Set(GB_JOINT_FREQUENCY, hz)) m_frequencyHz = hz; }
    void SetSpringDampingRatio(float ratio) { if (Set(GB_JOINT_DAMPING_RATIO, ratio)) m_dampingRatio = ratio; }
    bool IsMotorEnabled() const { return m_enableMotor; }
    float GetMotorSpeed() const { return m_motorSpeed; }
    float GetMaxMotorTorque() const { return m_maxMotorTorque; }
    float GetSpringFrequencyHz() const { return m_frequencyHz; }
    float GetSpringDampingRatio() const { return m_dampingRatio; }

private:
    friend class b2World;
    bool m_enableMotor = false;
    float m_motorSpeed = 0.0f, m_maxMotorTorque = 0.0f, m_frequencyHz = 0.0f, m_dampingRatio = 0.0f;
};
class b2DistanceJoint : public b2Joint {
public:
    void SetLength(float length) { if (Set(GB_JOINT_LENGTH, length)) m_length = length; }
    void SetFrequency(float hz) { if (Set(GB_JOINT_FREQUENCY, hz)) m_frequencyHz = hz; }
    void SetDampingRatio(float ratio) { if (Set(GB_JOINT_DAMPING_RATIO, ratio)) m_dampingRatio = ratio; }
    float GetLength() const { return m_length; }
    float GetFrequency() const { return m_frequencyHz; }
    float GetDampingRatio() const { return m_dampingRatio; }

private:
    friend class b2World;
    float m_length = 1.0f, m_frequencyHz = 0.0f, m_dampingRatio = 0.0f;
};
class b2WeldJoint : public b2Joint {
public:
    void SetFrequency(float hz) { if (Set(GB_JOINT_FREQUENCY, hz)) m_frequencyHz = hz; }
    void SetDampingRatio(float ratio) { if (Set(GB_JOINT_DAMPING_RATIO, ratio)) m_dampingRatio = ratio; }
    float GetFrequency() const { return m_frequencyHz; }
    float GetDampingRatio() const { return m_dampingRatio; }

private:
    friend class b2World;
    float m_frequencyHz = 0.0f, m_dampingRatio = 0.0f;
};
class b2RopeJoint : public b2Joint {
public:
    void SetMaxLength(float length) { if (Set(GB_JOINT_MAX_LENGTH, length)) m_maxLength = length; }
    float GetMaxLength() const { return m_maxLength; }

private:
    friend class b2World;
    float m_maxLength = 0.0f;
};
class b2FrictionJoint : public b2Joint {
public:
    void SetMaxForce(float force) { if (Set(GB_JOINT_MAX_FORCE, force)) m_maxForce = force; }
    void SetMaxTorque(float torque) { if (Set(GB_JOINT_MAX_TORQUE, torque)) m_maxTorque = torque; }
    float GetMaxForce() const { return m_maxForce; }
    float GetMaxTorque() const { return m_maxTorque; }

private:
    friend class b2World;
    float m_maxForce = 0.0f, m_maxTorque = 0.0f;
};
class b2MotorJoint : public b2Joint {
public:
    void SetLinearOffset(const b2Vec2& offset)
    {
        if (Set(GB_JOINT_LINEAR_OFFSET, offset.x, offset.y)) m_linearOffset = offset;
    }
    void SetAngularOffset(float offset) { if (Set(GB_JOINT_ANGULAR_OFFSET, offset)) m_angularOffset = offset; }
    void SetMaxForce(float force) { if (Set(GB_JOINT_MAX_FORCE, force)) m_maxForce = force; }
    void SetMaxTorque(float torque) { if (Set(GB_JOINT_MAX_TORQUE, torque)) m_maxTorque = torque; }
    void SetCorrectionFactor(float factor) { if (Set(GB_JOINT_CORRECTION_FACTOR, factor)) m_correctionFactor = factor; }
    const b2Vec2& GetLinearOffset() const { return m_linearOffset; }
    float GetAngularOffset() const { return m_angularOffset; }
    float GetMaxForce() const { return m_maxForce; }
    float GetMaxTorque() const { return m_maxTorque; }
    float GetCorrectionFactor() const { return m_correctionFactor; }

private:
    friend class b2World;
    b2Vec2 m_linearOffset;
    float m_angularOffset = 0.0f, m_maxForce = 0.0f, m_maxTorque = 0.0f, m_correctionFactor = 0.0f;
};
class b2GearJoint : public b2Joint {
public:
    void SetRatio(float ratio) { if (Set(GB_JOINT_RATIO, ratio)) m_ratio = ratio; }
    float GetRatio() const { return m_ratio; }

private:
    friend class b2World;
    float m_ratio = 1.0f;
};

// b2MouseJoint (Box2D/Dynamics/Joints/b2MouseJoint.h:63-124): what CreateJoint returns for a
// b2MouseJointDef, so the reference's static_cast<b2MouseJoint*> and SetTarget read the same.
class b2MouseJoint : public b2Joint {
public:
    void SetTarget(const b2Vec2& target);  // one gb_body_edits record (GB_EDIT_MOUSE_TARGET)
    const b2Vec2& GetTarget() const { return m_target; }
    void SetMaxForce(float force) { if (Set(GB_JOINT_MAX_FORCE, force)) m_maxForce = force; }
    void SetFrequency(float hz) { if (Set(GB_JOINT_FREQUENCY, hz)) m_frequencyHz = hz; }
    void SetDampingRatio(float ratio) { if (Set(GB_JOINT_DAMPING_RATIO, ratio)) m_dampingRatio = ratio; }
    float GetMaxForce() const { return m_maxForce; }
    float GetFrequency() const { return m_frequencyHz; }
    float GetDampingRatio() const { return m_dampingRatio; }

private:
    friend class b2World;
    b2Vec2 m_target;
    float m_maxForce = 0.0f, m_frequencyHz = 5.0f, m_dampingRatio = 0.7f;
};

struct b2ManifoldPoint {
    b2Vec2 localPoint;
    float normalImpulse = 0.0f, tangentImpulse = 0.0f;
    uint32_t id = 0;
};
struct b2Manifold {
    enum Type { e_circles = 0, e_faceA = 1, e_faceB = 2 };
    b2ManifoldPoint points[2];
    b2Vec2 localNormal, localPoint;
    Type type = e_circles;
    int pointCount = 0;
};

// b2WorldManifold (Box2D/Collision/b2Collision.h:115-126) and its Initialize (b2Collision.cpp:25-66):
// the world normal (A to B), contact points (midway between the surfaces) and separations.
struct b2WorldManifold {
    b2Vec2 normal;
    b2Vec2 points[2];
    float separations[2] = {0.0f, 0.0f};
    void Initialize(const b2Manifold* manifold, const b2Transform& xfA, float radiusA, const b2Transform& xfB,
                    float radiusB)
    {
        if (manifold->pointCount == 0) return;
        auto mul = [](const b2Transform& t, const b2Vec2& v) {
            return b2Vec2((t.q.c * v.x - t.q.s * v.y) + t.p.x, (t.q.s * v.x + t.q.c * v.y) + t.p.y);
        };
        auto rot = [](const b2Transform& t, const b2Vec2& v) {
            return b2Vec2(t.q.c * v.x - t.q.s * v.y, t.q.s * v.x + t.q.c * v.y);
        };
        auto dot = [](const b2Vec2& a, const b2Vec2& b) { return a.x * b.x + a.y * b.y; };
        switch (manifold->type) {
        case b2Manifold::e_circles: {
            normal = b2Vec2(1.0f, 0.0f);
            const b2Vec2 pointA = mul(xfA, manifold->localPoint);
            const b2Vec2 pointB = mul(xfB, manifold->points[0].localPoint);
            const b2Vec2 d(pointA.x - pointB.x, pointA.y - pointB.y);
            const float eps = 1.19209289550781250e-7f;  // FLT_EPSILON
            if (dot(d, d) > eps * eps) {
                normal = b2Vec2(pointB.x - pointA.x, pointB.y - pointA.y);
                const float length = std::sqrt(normal.x * normal.x + normal.y * normal.y);
                if (length >= eps) {
                    const float inv = 1.0f / length;
                    normal.x *= inv;
                    normal.y *= inv;
                }
            }
            const b2Vec2 cA(pointA.x + radiusA * normal.x, pointA.y + radiusA * normal.y);
            const b2Vec2 cB(pointB.x - radiusB * normal.x, pointB.y - radiusB * normal.y);
            points[0] = b2Vec2(0.5f * (cA.x + cB.x), 0.5f * (cA.y + cB.y));
            separations[0] = dot(b2Vec2(cB.x - cA.x, cB.y - cA.y), normal);
        } break;
        case b2Manifold::e_faceA: {
            normal = rot(xfA, manifold->localNormal);
            const b2Vec2 planePoint = mul(xfA, manifold->localPoint);
            for (int i = 0; i < manifold->pointCount; ++i) {
                const b2Vec2 clip = mul(xfB, manifold->points[i].localPoint);
                const float s = radiusA - dot(b2Vec2(clip.x - planePoint.x, clip.y - planePoint.y), normal);
                const b2Vec2 cA(clip.x + s * normal.x, clip.y + s * normal.y);
                const b2Vec2 cB(clip.x - radiusB * normal.x, clip.y - radiusB * normal.y);
                points[i] = b2Vec2(0.5f * (cA.x + cB.x), 0.5f * (cA.y + cB.y));
                separations[i] = dot(b2Vec2(cB.x - cA.x, cB.y - cA.y), normal);
            }
        } break;
        case b2Manifold::e_faceB: {
            normal = rot(xfB, manifold->localNormal);
            const b2Vec2 planePoint = mul(xfB, manifold->localPoint);
            for (int i = 0; i < manifold->pointCount; ++i) {
                const b2Vec2 clip = mul(xfA, manifold->points[i].localPoint);
                const float s = radiusB - dot(b2Vec2(clip.x - planePoint.x, clip.y - planePoint.y), normal);
                const b2Vec2 cB(clip.x + s * normal.x, clip.y + s * normal.y);
                const b2Vec2 cA(clip.x - radiusA * normal.x, clip.y - radiusA * normal.y);
                points[i] = b2Vec2(0.5f * (cA.x + cB.x), 0.5f * (cA.y + cB.y));
                separations[i] = dot(b2Vec2(cA.x - cB.x, cA.y - cB.y), normal);
            }
            normal = b2Vec2(-normal.x, -normal.y);
        } break;
        }
    }
};

class b2Contact {
public:
    b2Fixture* GetFixtureA() const { return m_a; }
    b2Fixture* GetFixtureB() const { return m_b; }
    int GetChildIndexA() const { return m_childA; }  // the chain child, 0 for other shapes
    int GetChildIndexB() const { return m_childB; }
    bool IsTouching() const { return (m_flags & 2) != 0; }
    // the next contact of the world's list (b2Contact::GetNext), valid until the next step
    b2Contact* GetNext() { return m_next; }
    const b2Contact* GetNext() const { return m_next; }
    bool IsEnabled() const { return (m_flags & 4) != 0; }
    // b2Contact::SetEnabled, SetFriction, SetRestitution, SetTangentSpeed (Contacts/b2Contact.h:98-152),
    // in effect for the rest of a step when made in PreSolve
    void SetEnabled(bool flag)
    {
        m_flags = flag ? (m_flags | 4) : (m_flags & ~4);
        m_edit |= 1;
    }
    void SetFriction(float friction) { m_friction = friction; m_edit |= 2; }
    void SetRestitution(float restitution) { m_restitution = restitution; m_edit |= 4; }
    void SetTangentSpeed(float speed) { m_tangentSpeed = speed; m_edit |= 8; }
    const b2Manifold* GetManifold() const { return &m_manifold; }
    // b2Contact::GetWorldManifold (Box2D/Dynamics/Contacts/b2Contact.h:223-231)
    void GetWorldManifold(b2WorldManifold* worldManifold) const;

private:
    friend class b2World;
    b2Fixture *m_a = nullptr, *m_b = nullptr;
    int m_childA = 0, m_childB = 0;
    int m_idA = -1, m_idB = -1;  // device fixture ids (one per chain child)
    int m_flags = 0;
    int m_edit = 0;               // changes made by the listener (gb_contact_edit flags)
    b2Contact* m_next = nullptr;  // the next contact of the world's list
    float m_friction = 0.0f, m_restitution = 0.0f, m_tangentSpeed = 0.0f;
    b2Manifold m_manifold;
};

struct b2ContactImpulse {
    float normalImpulses[2] = {0.0f, 0.0f};
    float tangentImpulses[2] = {0.0f, 0.0f};
    int count = 0;
};

class b2ContactListener {
public:
    virtual ~b2ContactListener() = default;
    virtual void BeginContact(b2Contact*) {}
    virtual void EndContact(b2Contact*) {}
    virtual void PreSolve(b2Contact*, const b2Manifold*) {}
    virtual void PostSolve(b2Contact*, const b2ContactImpulse*) {}
};

// b2DestructionListener, b2QueryCallback, b2RayCastCallback (Box2D/Dynamics/b2WorldCallbacks.h:38-155)
class b2DestructionListener {
public:
    virtual ~b2DestructionListener() = default;
    virtual void SayGoodbye(b2Joint* joint) = 0;
    virtual void SayGoodbye(b2Fixture* fixture) = 0;
};
// b2ContactFilter (Box2D/Dynamics/b2WorldCallbacks.h:52-63); the default is category/mask/group
// (b2WorldCallbacks.cpp:26-38)
class b2ContactFilter {
public:
    virtual ~b2ContactFilter() = default;
    virtual bool ShouldCollide(b2Fixture* fixtureA, b2Fixture* fixtureB)
    {
        const b2Filter& a = fixtureA->GetFilterData();
        const b2Filter& b = fixtureB->GetFilterData();
        if (a.groupIndex == b.groupIndex && a.groupIndex != 0) return a.groupIndex > 0;
        return (a.maskBits & b.categoryBits) != 0 && (a.categoryBits & b.maskBits) != 0;
    }
};
class b2QueryCallback {
public:
    virtual ~b2QueryCallback() = default;
    virtual bool ReportFixture(b2Fixture* fixture) = 0;
};
class b2RayCastCallback {
public:
    virtual ~b2RayCastCallback() = default;
    virtual float ReportFixture(b2Fixture* fixture, const b2Vec2& point, const b2Vec2& normal, float fraction) = 0;
};

// b2Profile (Box2D/Dynamics/b2TimeStep.h:27-37), milliseconds of the device step
struct b2Profile {
    float step = 0, collide = 0, solve = 0, solveInit = 0, solveVelocity = 0, solvePosition = 0, broadphase = 0,
          solveTOI = 0;
};

class b2World {
public:
    explicit b2World(const b2Vec2& gravity) : m_gravity(gravity) {}
    ~b2World()
    {
        if (m_h) gb_world_destroy(m_h);
    }
    b2World(const b2World&) = delete;
    b2World& operator=(const b2World&) = delete;

    // the world settings (Box2D/Dynamics/b2World.h:145-217): kept here and, once the device world
    // exists, applied to it between steps (gb_world_set_settings)
    void SetAllowSleeping(bool flag) { m_def.allow_sleep = flag; ApplySettings(); }
    void SetWarmStarting(bool flag) { m_def.warm_starting = flag; ApplySettings(); }
    void SetContinuousPhysics(bool flag) { m_def.continuous_physics = flag; ApplySettings(); }
    void SetSubStepping(bool flag) { m_def.sub_stepping = flag; ApplySettings(); }
    void SetGravity(const b2Vec2& gravity) { m_gravity = gravity; ApplySettings(); }
    void SetAutoClearForces(bool flag) { m_autoClear = flag; ApplySettings(); }
    bool GetAllowSleeping() const { return m_def.allow_sleep != 0; }
    // b2World::IsLocked (Box2D/Dynamics/b2World.h:169): true while the contact listener is being called
    bool IsLocked() const { return m_locked; }
    bool GetWarmStarting() const { return m_def.warm_starting != 0; }
    bool GetContinuousPhysics() const { return m_def.continuous_physics != 0; }
    bool GetSubStepping() const { return m_def.sub_stepping != 0; }
    bool GetAutoClearForces() const { return m_autoClear; }
    b2Vec2 GetGravity() const { return m_gravity; }
    // b2World::ClearForces (Box2D/Dynamics/b2World.cpp:967-974)
    void ClearForces()
    {
        if (m_h) gb_world_clear_forces(m_h, 0);
    }
    void SetContactListener(b2ContactListener* listener) { m_listener = listener; }
    void SetDestructionListener(b2DestructionListener* listener) { m_destruction = listener; }
    // b2World::SetContactFilter (Box2D/Dynamics/b2World.cpp:94): the filter decides each ordered
    // fixture pair once (see gb_world_set_contact_filter); with a filter set, Step runs whole (a
    // PreSolve listener is then notified only)
    void SetContactFilter(b2ContactFilter* filter)
    {
        m_filter = filter;
        if (!Handle()) return;
        gb_world_set_contact_filter(m_h, filter ? &b2World::FilterTrampoline : nullptr, this);
    }

    // b2World::DestroyBody (Box2D/Dynamics/b2World.cpp:133-212)
    void DestroyBody(b2Body* body)
    {
        if (!m_h || !body || !body->m_alive || body->m_world != this) return;
        std::vector<int> calls;
        if (Destroy(gb_destroy_body, body->m_index, calls) != GB_OK) return;
        body->m_alive = false;
        Announce(calls);
        for (auto& f : m_fixtures)
            if (f->m_body == body) f->m_alive = false;
    }
    // b2World::DestroyJoint (Box2D/Dynamics/b2World.cpp:274-362)
    void DestroyJoint(b2Joint* joint)
    {
        if (!m_h || !joint || !joint->m_alive || joint->m_world != this) return;
        std::vector<int> calls;
        if (Destroy(gb_destroy_joint, joint->m_index, calls) != GB_OK) return;
        joint->m_alive = false;
    }
    // one gb_fixture_query call (b2Fixture::TestPoint, RayCast, GetAABB)
    bool FixtureQuery(int index, int op, const float* in, float* out)
    {
        out[0] = out[1] = out[2] = out[3] = 0.0f;
        return Handle() && gb_fixture_query(m_h, 0, index, op, in, out) == GB_OK;
    }
    // a joint's reaction force and torque (gb_get_joint_reaction)
    void JointReaction(int index, float inv_dt, float* out)
    {
        out[0] = out[1] = out[2] = 0.0f;
        if (Handle()) gb_get_joint_reaction(m_h, 0, index, inv_dt, out);
    }
    // one gb_joint_set call (the typed joints' setters)
    bool SetJointProperty(b2Joint* j, int prop, float v0, float v1)
    {
        if (!Handle() || !j || !j->m_alive || j->m_world != this) return false;
        const float v[4] = {v0, v1, 0.0f, 0.0f};
        MarkStale();
        return gb_joint_set(m_h, 0, j->m_index, prop, v) == GB_OK;
    }
    // b2World::ShiftOrigin (Box2D/Dynamics/b2World.cpp:1261-1282)
    void ShiftOrigin(const b2Vec2& newOrigin)
    {
        if (!Handle()) return;
        gb_world_shift_origin(m_h, 0, newOrigin.x, newOrigin.y);
        MarkStale();
    }
    // one gb_fixture_set call (b2Fixture::SetFriction, ...)
    bool SetFixtureProperty(b2Fixture* f, int prop, float v0, float v1 = 0.0f, float v2 = 0.0f)
    {
        if (!Handle() || !f || !f->m_alive) return false;
        const float v[4] = {v0, v1, v2, 0.0f};
        MarkStale();
        return gb_fixture_set(m_h, 0, f->m_index, prop, v) == GB_OK;
    }
    // one gb_body_set call (b2Body::SetType, SetActive, ...); EndContact for the contacts it destroys
    bool SetBodyProperty(b2Body* body, int prop, float value, float v1 = 0.0f, float v2 = 0.0f, float v3 = 0.0f)
    {
        if (!Handle() || !body || !body->m_alive || body->m_world != this) return false;
        if (m_listener) ReadContacts();  // the contacts an EndContact may name
        const int cap = GetContactCount() + 1;
        std::vector<int> calls(3 * (size_t)cap, 0);
        int n = 0;
        const float v[4] = {value, v1, v2, v3};
        const gb_status s = gb_body_set(m_h, 0, body->m_index, prop, v, calls.data(), cap, &n);
        MarkStale();
        if (s != GB_OK) return false;
        calls.resize(3 * (size_t)std::min(n, cap));
        Announce(calls);
        return true;
    }
    void DestroyFixture(b2Fixture* fixture)
    {
        if (!m_h || !fixture || !fixture->m_alive) return;
        std::vector<int> calls;
        if (Destroy(gb_destroy_fixture, fixture->m_index, calls) != GB_OK) return;
        fixture->m_alive = false;
        Announce(calls);
    }

    // b2World::QueryAABB (Box2D/Dynamics/b2World.cpp:988-994): each fixture proxy whose fat AABB
    // overlaps the box, until the callback returns false
    void QueryAABB(b2QueryCallback* callback, const b2AABB& aabb)
    {
        if (!Handle() || !callback) return;
        const float box[4] = {aabb.lowerBound.x, aabb.lowerBound.y, aabb.upperBound.x, aabb.upperBound.y};
        int offsets[2] = {0, 0}, total = 0;
        gb_world_query_aabb(m_h, 0, 1, box, offsets, nullptr, 0, &total);
        std::vector<int> ids((size_t)(total > 0 ? total : 1));
        if (total > 0 && gb_world_query_aabb(m_h, 0, 1, box, offsets, ids.data(), total, &total) != GB_OK) return;
        for (int k = 0; k < total; ++k)
            if (!callback->ReportFixture(m_fixtureOfId[ids[k]].first)) return;
    }
    // b2World::RayCast (Box2D/Dynamics/b2World.cpp:1021-1035) and b2DynamicTree::RayCast's use of the
    // callback's value (b2DynamicTree.h:218-280)
    void RayCast(b2RayCastCallback* callback, const b2Vec2& point1, const b2Vec2& point2)
    {
        if (!Handle() || !callback) return;
        const float ray[4] = {point1.x, point1.y, point2.x, point2.y};
        const int cap = (int)m_fixtureOfId.size();
        std::vector<int> ids((size_t)(cap > 0 ? cap : 1));
        std::vector<float> hits(5 * (size_t)(cap > 0 ? cap : 1));
        int n = 0;
        if (gb_world_raycast_all(m_h, 0, ray, ids.data(), hits.data(), cap, &n) != GB_OK) return;
        float maxFraction = 1.0f;
        for (int k = 0; k < n; ++k) {
            const float* h = &hits[5 * (size_t)k];
            if (h[0] > maxFraction) continue;  // beyond the clipped ray: the fixture reports no hit
            const float value = callback->ReportFixture(m_fixtureOfId[ids[k]].first, b2Vec2(h[1], h[2]),
                                                        b2Vec2(h[3], h[4]), h[0]);
            if (value == 0.0f) return;
            if (value > 0.0f) maxFraction = value;
        }
    }

    // b2World::GetBodyList (newest first, as the reference's list)
    b2Body* GetBodyList() const { return PreviousAlive(m_bodies.size()); }
    // b2World::GetJointList (newest first)
    b2Joint* GetJointList() const { return PreviousJoint(m_joints.size()); }
    b2Joint* PreviousJoint(size_t slot) const
    {
        for (size_t i = slot; i-- > 0;)
            if (m_joints[i]->m_alive) return m_joints[i].get();
        return nullptr;
    }
    b2Fixture* FixtureListOf(const b2Body* body) const { return PreviousFixture(m_fixtures.size(), body); }
    // a body's fixtures before `slot` in creation order, newest first (b2Body::GetFixtureList order)
    b2Fixture* PreviousFixture(size_t slot, const b2Body* body) const
    {
        for (size_t i = slot; i-- > 0;)
            if (m_fixtures[i]->m_alive && m_fixtures[i]->m_body == body) return m_fixtures[i].get();
        return nullptr;
    }
    b2Body* PreviousAlive(size_t index) const
    {
        for (size_t i = index; i-- > 0;)
            if (m_bodies[i]->m_alive) return m_bodies[i].get();
        return nullptr;
    }
    // b2World::GetProxyCount (Box2D/Dynamics/b2World.cpp:1241): broadphase proxies (one per chain child)
    int GetProxyCount()
    {
        if (!Handle() || m_fixtureOfId.empty()) return 0;
        std::vector<int> ids(m_fixtureOfId.size());
        if (gb_get_proxies(m_h, 0, ids.data(), nullptr) != GB_OK) return 0;
        int n = 0;
        for (int id : ids) n += id >= 0 ? 1 : 0;
        return n;
    }
    // b2World::GetTreeHeight, GetTreeBalance, GetTreeQuality (Box2D/Dynamics/b2World.cpp:1246-1259): the
    // broadphase tree the world replays on the host (0 when it cannot)
    int GetTreeHeight()
    {
        int h = 0;
        if (!Handle() || gb_world_tree_stats(m_h, 0, &h, nullptr, nullptr) != GB_OK) return 0;
        return h;
    }
    int GetTreeBalance()
    {
        int b = 0;
        if (!Handle() || gb_world_tree_stats(m_h, 0, nullptr, &b, nullptr) != GB_OK) return 0;
        return b;
    }
    float GetTreeQuality()
    {
        float q = 0.0f;
        if (!Handle() || gb_world_tree_stats(m_h, 0, nullptr, nullptr, &q) != GB_OK) return 0.0f;
        return q;
    }
    // b2World::GetProfile (Box2D/Dynamics/b2World.h:196) of the last step
    const b2Profile& GetProfile()
    {
        float ms[8] = {0};
        if (m_h) gb_world_get_profile(m_h, 0, ms);
        m_profile.step = ms[0]; m_profile.collide = ms[1]; m_profile.solve = ms[2]; m_profile.solveInit = ms[3];
        m_profile.solveVelocity = ms[4]; m_profile.solvePosition = ms[5]; m_profile.broadphase = ms[6];
        m_profile.solveTOI = ms[7];
        return m_profile;
    }

    b2Body* CreateBody(const b2BodyDef* def)
    {
        if (!Handle()) return nullptr;
        const float f[9] = {def->position.x, def->position.y, def->angle, def->linearVelocity.x, def->linearVelocity.y,
                            def->angularVelocity, def->linearDamping, def->angularDamping, def->gravityScale};
        const int flags = (def->allowSleep ? 1 : 0) | (def->awake ? 2 : 0) | (def->fixedRotation ? 4 : 0) |
                          (def->bullet ? 8 : 0) | (def->active ? 16 : 0);
        const int type = def->type;
        int id = -1;
        if (gb_create_bodies(m_h, 0, 1, &type, f, &flags, &id) != GB_OK) return nullptr;
        std::unique_ptr<b2Body> b(new b2Body());
        b->m_world = this;
        b->m_index = id;
        b->m_type = def->type;
        b->m_userData = def->userData;
        m_bodies.push_back(std::move(b));
        MarkStale();
        return m_bodies.back().get();
    }

    b2Joint* CreateJoint(const b2RevoluteJointDef* def)
    {
        if (!Handle() || !def->bodyA || !def->bodyB) return nullptr;
        const float f[9] = {def->localAnchorA.x, def->localAnchorA.y, def->localAnchorB.x, def->localAnchorB.y,
                            def->referenceAngle, def->lowerAngle, def->upperAngle, def->motorSpeed,
                            def->maxMotorTorque};
        const int flags = (def->enableLimit ? 1 : 0) | (def->enableMotor ? 2 : 0) | (def->collideConnected ? 4 : 0);
        const int a = def->bodyA->m_index, b = def->bodyB->m_index;
        int id = -1;
        if (gb_create_revolute_joints(m_h, 0, 1, &a, &b, f, &flags, &id) != GB_OK) return nullptr;
        std::unique_ptr<b2RevoluteJoint> j(new b2RevoluteJoint());
        j->m_enableMotor = def->enableMotor;
        j->m_enableLimit = def->enableLimit;
        j->m_motorSpeed = def->motorSpeed;
        j->m_maxMotorTorque = def->maxMotorTorque;
        j->m_lower = def->lowerAngle;
        j->m_upper = def->upperAngle;
        j->m_world = this;
        j->m_index = id;
        j->m_a = def->bodyA;
        j->m_b = def->bodyB;
        j->m_userData = def->userData;
        j->m_slot = m_joints.size();
        m_joints.push_back(std::move(j));
        return m_joints.back().get();
    }

    b2Joint* CreateJoint(const b2DistanceJointDef* def)
    {
        const float f[GB_JOINT_FLOATS] = {def->localAnchorA.x, def->localAnchorA.y, def->localAnchorB.x,
                                          def->localAnchorB.y, def->length, def->frequencyHz, def->dampingRatio};
        std::unique_ptr<b2DistanceJoint> j(new b2DistanceJoint());
        j->m_length = def->length;
        j->m_frequencyHz = def->frequencyHz;
        j->m_dampingRatio = def->dampingRatio;
        b2Joint* r = AddJoint(GB_JOINT_DISTANCE, def->bodyA, def->bodyB, f, def->collideConnected ? 4 : 0, std::move(j));
        if (r) r->m_userData = def->userData;
        return r;
    }
    b2Joint* CreateJoint(const b2WeldJointDef* def)
    {
        const float f[GB_JOINT_FLOATS] = {def->localAnchorA.x, def->localAnchorA.y, def->localAnchorB.x,
                                          def->localAnchorB.y, def->referenceAngle, def->frequencyHz,
                                          def->dampingRatio};
        std::unique_ptr<b2WeldJoint> j(new b2WeldJoint());
        j->m_frequencyHz = def->frequencyHz;
        j->m_dampingRatio = def->dampingRatio;
        b2Joint* r = AddJoint(GB_JOINT_WELD, def->bodyA, def->bodyB, f, def->collideConnected ? 4 : 0, std::move(j));
        if (r) r->m_userData = def->userData;
        return r;
    }
    b2Joint* CreateJoint(const b2WheelJointDef* def)
    {
        const float f[GB_JOINT_FLOATS] = {def->localAnchorA.x, def->localAnchorA.y, def->localAnchorB.x,
                                          def->localAnchorB.y, def->localAxisA.x, def->localAxisA.y,
                                          def->maxMotorTorque, def->motorSpeed, def->frequencyHz, def->dampingRatio};
        const int flags = (def->enableMotor ? 2 : 0) | (def->collideConnected ? 4 : 0);
        std::unique_ptr<b2WheelJoint> j(new b2WheelJoint());
        j->m_enableMotor = def->enableMotor;
        j->m_motorSpeed = def->motorSpeed;
        j->m_maxMotorTorque = def->maxMotorTorque;
        j->m_frequencyHz = def->frequencyHz;
        j->m_dampingRatio = def->dampingRatio;
        b2Joint* r = AddJoint(GB_JOINT_WHEEL, def->bodyA, def->bodyB, f, flags, std::move(j));
        if (r) r->m_userData = def->userData;
        return r;
    }
    b2Joint* CreateJoint(const b2RopeJointDef* def)
    {
        const float f[GB_JOINT_FLOATS] = {def->localAnchorA.x, def->localAnchorA.y, def->localAnchorB.x,
                                          def->localAnchorB.y, def->maxLength};
        std::unique_ptr<b2RopeJoint> j(new b2RopeJoint());
        j->m_maxLength = def->maxLength;
        b2Joint* r = AddJoint(GB_JOINT_ROPE, def->bodyA, def->bodyB, f, def->collideConnected ? 4 : 0, std::move(j));
        if (r) r->m_userData = def->userData;
        return r;
    }
    b2Joint* CreateJoint(const b2FrictionJointDef* def)
    {
        const float f[GB_JOINT_FLOATS] = {def->localAnchorA.x, def->localAnchorA.y, def->localAnchorB.x,
                                          def->localAnchorB.y, def->maxForce, def->maxTorque};
        std::unique_ptr<b2FrictionJoint> j(new b2FrictionJoint());
        j->m_maxForce = def->maxForce;
        j->m_maxTorque = def->maxTorque;
        b2Joint* r = AddJoint(GB_JOINT_FRICTION, def->bodyA, def->bodyB, f, def->collideConnected ? 4 : 0, std::move(j));
        if (r) r->m_userData = def->userData;
        return r;
    }
    b2Joint* CreateJoint(const b2MotorJointDef* def)
    {
        const float f[GB_JOINT_FLOATS] = {def->linearOffset.x, def->linearOffset.y, def->angularOffset, def->maxForce,
                                          def->maxTorque, def->correctionFactor};
        std::unique_ptr<b2MotorJoint> j(new b2MotorJoint());
        j->m_linearOffset = def->linearOffset;
        j->m_angularOffset = def->angularOffset;
        j->m_maxForce = def->maxForce;
        j->m_maxTorque = def->maxTorque;
        j->m_correctionFactor = def->correctionFactor;
        b2Joint* r = AddJoint(GB_JOINT_MOTOR, def->bodyA, def->bodyB, f, def->collideConnected ? 4 : 0, std::move(j));
        if (r) r->m_userData = def->userData;
        return r;
    }
    b2Joint* CreateJoint(const b2MouseJointDef* def)
    {
        const float f[GB_JOINT_FLOATS] = {def->target.x, def->target.y, def->maxForce, def->frequencyHz,
                                          def->dampingRatio};
        std::unique_ptr<b2MouseJoint> j(new b2MouseJoint());
        j->m_target = def->target;
        j->m_maxForce = def->maxForce;
        j->m_frequencyHz = def->frequencyHz;
        j->m_dampingRatio = def->dampingRatio;
        b2Joint* r = AddJoint(GB_JOINT_MOUSE, def->bodyA, def->bodyB, f, def->collideConnected ? 4 : 0, std::move(j));
        if (r) r->m_userData = def->userData;
        return r;
    }
    b2Joint* CreateJoint(const b2PulleyJointDef* def)
    {
        const float f[GB_JOINT_FLOATS] = {def->groundAnchorA.x, def->groundAnchorA.y, def->groundAnchorB.x,
                                          def->groundAnchorB.y, def->localAnchorA.x, def->localAnchorA.y,
                                          def->localAnchorB.x, def->localAnchorB.y, def->lengthA, def->lengthB,
                                          def->ratio};
        b2Joint* r = AddJoint(GB_JOINT_PULLEY, def->bodyA, def->bodyB, f, def->collideConnected ? 4 : 0);
        if (r) r->m_userData = def->userData;
        return r;
    }
    b2Joint* CreateJoint(const b2GearJointDef* def)
    {
        if (!def->joint1 || !def->joint2) return nullptr;
        const float f[GB_JOINT_FLOATS] = {(float)def->joint1->GetIndex(), (float)def->joint2->GetIndex(), def->ratio};
        std::unique_ptr<b2GearJoint> g(new b2GearJoint());
        g->m_ratio = def->ratio;
        b2Joint* j = AddJoint(GB_JOINT_GEAR, def->bodyA, def->bodyB, f, def->collideConnected ? 4 : 0, std::move(g));
        if (j) j->m_userData = def->userData;
        if (j) {  // b2GearJoint::GetBodyA/B: the coupled joints' bodies B
            j->m_a = def->joint1->GetBodyB();
            j->m_b = def->joint2->GetBodyB();
        }
        return j;
    }
    b2Joint* CreateJoint(const b2PrismaticJointDef* def)
    {
        const float f[GB_JOINT_FLOATS] = {def->localAnchorA.x, def->localAnchorA.y, def->localAnchorB.x,
                                          def->localAnchorB.y, def->localAxisA.x, def->localAxisA.y,
                                          def->referenceAngle, def->lowerTranslation, def->upperTranslation,
                                          def->maxMotorForce, def->motorSpeed};
        const int flags = (def->enableLimit ? 1 : 0) | (def->enableMotor ? 2 : 0) | (def->collideConnected ? 4 : 0);
        std::unique_ptr<b2PrismaticJoint> j(new b2PrismaticJoint());
        j->m_enableMotor = def->enableMotor;
        j->m_enableLimit = def->enableLimit;
        j->m_motorSpeed = def->motorSpeed;
        j->m_maxMotorForce = def->maxMotorForce;
        j->m_lower = def->lowerTranslation;
        j->m_upper = def->upperTranslation;
        b2Joint* r = AddJoint(GB_JOINT_PRISMATIC, def->bodyA, def->bodyB, f, flags, std::move(j));
        if (r) r->m_userData = def->userData;
        return r;
    }

    void Step(float timeStep, int velocityIterations, int positionIterations)
    {
        if (!Handle()) return;
        if (!m_listener) {
            gb_world_step(m_h, timeStep, velocityIterations, positionIterations);
            MarkStale();
            return;
        }
        if (m_filter) {
            if (!m_eventsOn) m_eventsOn = gb_world_set_events(m_h, 1) == GB_OK;
            ReadContacts();
            gb_world_step(m_h, timeStep, velocityIterations, positionIterations);
            MarkStale();
            Report(0);
            return;
        }
        if (!m_eventsOn) m_eventsOn = gb_world_set_events(m_h, 1) == GB_OK;
        ReadContacts();  // the contacts before the step: destroyed contacts and old manifolds
        if (gb_world_step_begin(m_h, timeStep, velocityIterations, positionIterations) != GB_OK) return;
        MarkStale();
        const int collideCalls = Report(0);
        // what PreSolve changed, by list position
        std::vector<gb_contact_edit> edits;
        for (size_t k = 0; k < m_contacts.size(); ++k) {
            const b2Contact& c = *m_contacts[k];
            if (!c.m_edit) continue;
            gb_contact_edit e{0, (int)k, c.m_edit, c.IsEnabled() ? 1 : 0, c.m_friction, c.m_restitution,
                              c.m_tangentSpeed, 0.0f};
            edits.push_back(e);
        }
        if (!edits.empty()) gb_contact_edits(m_h, (int)edits.size(), edits.data());
        gb_world_step_end(m_h);
        MarkStale();
        Report(collideCalls);
    }

    int GetBodyCount() const
    {
        int n = 0;
        for (const auto& b : m_bodies) n += b->m_alive ? 1 : 0;
        return n;
    }
    int GetJointCount() const
    {
        int n = 0;
        for (const auto& j : m_joints) n += j->m_alive ? 1 : 0;
        return n;
    }
    int GetContactCount()
    {
        int b = 0, f = 0, c = 0, j = 0;
        if (m_h) gb_world_counts(m_h, 0, &b, &f, &c, &j);
        return c;
    }
    // b2World::GetContactList (Box2D/Dynamics/b2World.h:127): the head of the world's contact list
    // (newest first; b2Contact::GetNext walks it), read once after each step or change
    b2Contact* GetContactList()
    {
        const std::vector<b2Contact*>& v = Contacts();
        return v.empty() ? nullptr : v[0];
    }
    // the same list as a vector; the contacts stay the same objects until the next step or change
    const std::vector<b2Contact*>& Contacts()
    {
        if (!m_contactsStale && !m_contactView.empty()) return m_contactView;
        // inside the listener's calls the list is the one being reported (read at this half's end)
        if (!m_locked) {
            ReadContacts();
            m_contactsStale = false;
        }
        m_contactView.clear();
        for (auto& c : m_contacts) m_contactView.push_back(c.get());
        return m_contactView;
    }

    // the body states and the contact list are read again at their next use
    void MarkStale()
    {
        m_stale = true;
        m_contactsStale = true;
    }
    // raw access used by b2Body
    // a body's mass data, damping and flags (gb_get_body_info), for the b2Body getters
    int BodyInfo(int index, float* out)
    {
        int flags = 0;
        if (!Handle() || gb_get_body_info(m_h, 0, index, out, &flags) != GB_OK) return 0;
        return flags;
    }
    const float* BodyState(int index)
    {
        if (m_stale) {
            m_state.assign(12 * m_bodies.size(), 0.0f);
            if (!m_bodies.empty()) gb_get_bodies(m_h, 0, m_state.data());
            m_stale = false;
        }
        return m_state.data() + 12 * index;
    }
    b2Fixture* AddFixture(b2Body* body, const b2FixtureDef* def)
    {
        if (!Handle() || !def->shape) return nullptr;
        int type = 0, n = 0;
        float shape[16] = {0};
        def->shape->Encode(&type, shape, &n);
        const float mat[3] = {def->density, def->friction, def->restitution};
        const int filt[4] = {def->filter.categoryBits, def->filter.maskBits, def->filter.groupIndex, def->isSensor ? 1 : 0};
        const int b = body->GetIndex();
        int id = -1, children = 1;
        if (def->shape->GetType() == b2Shape::e_chain) {
            const b2ChainShape* chain = static_cast<const b2ChainShape*>(def->shape);
            std::vector<float> xy;
            for (const b2Vec2& v : chain->m_vertices) { xy.push_back(v.x); xy.push_back(v.y); }
            const float pn[4] = {chain->m_prevVertex.x, chain->m_prevVertex.y, chain->m_nextVertex.x,
                                 chain->m_nextVertex.y};
            const int ghosts = (chain->m_hasPrevVertex ? 1 : 0) | (chain->m_hasNextVertex ? 2 : 0);
            if (gb_create_chain(m_h, 0, b, xy.data(), (int)chain->m_vertices.size(), chain->m_loop ? 1 : 0, pn,
                                ghosts, mat, filt, &id) != GB_OK)
                return nullptr;
            children = chain->GetChildCount();
        } else if (gb_create_fixtures(m_h, 0, 1, &b, &type, shape, &n, mat, filt, &id) != GB_OK) {
            return nullptr;
        }
        std::unique_ptr<b2Fixture> fx(new b2Fixture());
        fx->m_body = body;
        fx->m_index = id;
        fx->m_def = *def;
        fx->m_def.shape = nullptr;
        fx->m_type = def->shape->GetType();
        fx->m_radius = def->shape->m_radius;
        for (int k = 0; k < children; ++k) m_fixtureOfId.push_back({fx.get(), k});
        fx->m_slot = m_fixtures.size();
        m_fixtures.push_back(std::move(fx));
        MarkStale();
        return m_fixtures.back().get();
    }
    void Edit(int index, int op, float v0, float v1, float v2, float v3, bool wake)
    {
        if (!Handle()) return;
        gb_body_edit e;
        e.world = 0;
        e.body = index;
        e.op = op;
        e.wake = wake ? 1 : 0;
        e.v[0] = v0; e.v[1] = v1; e.v[2] = v2; e.v[3] = v3;
        gb_body_edits(m_h, 1, &e);
        MarkStale();
    }

private:
    static int FilterTrampoline(void* user, int, int fixtureA, int fixtureB)
    {
        b2World* self = static_cast<b2World*>(user);
        return self->m_filter->ShouldCollide(self->m_fixtureOfId[fixtureA].first, self->m_fixtureOfId[fixtureB].first)
                   ? 1
                   : 0;
    }
    // one gb_destroy_* call; its listener calls in calls (3 ints each)
    gb_status Destroy(gb_status (*fn)(gb_world*, int, int, int*, int, int*), int index, std::vector<int>& calls)
    {
        if (m_listener) ReadContacts();  // the contacts an EndContact may name
        // room for every call the destruction can make: each joint, contact and fixture of the world
        const int cap = GetContactCount() + (int)m_joints.size() + (int)m_fixtureOfId.size() + 1;
        int n = 0;
        calls.assign(3 * (size_t)cap, 0);
        gb_status s = fn(m_h, 0, index, calls.data(), cap, &n);
        calls.resize(3 * (size_t)(s == GB_OK ? std::min(n, cap) : 0));
        MarkStale();
        return s;
    }
    void Announce(const std::vector<int>& calls)
    {
        for (size_t k = 0; k + 2 < calls.size(); k += 3) {
            const int kind = calls[k], a = calls[k + 1], b = calls[k + 2];
            if (kind == 0) {
                for (auto& j : m_joints)
                    if (j->m_index == a) {
                        j->m_alive = false;
                        if (m_destruction) m_destruction->SayGoodbye(j.get());
                    }
            } else if (kind == 1) {
                if (m_destruction) m_destruction->SayGoodbye(m_fixtureOfId[a].first);
            } else if (m_listener) {
                for (auto& c : m_contacts)
                    if (c->m_idA == a && c->m_idB == b) m_listener->EndContact(c.get());
            }
        }
    }
    b2Joint* AddJoint(int type, b2Body* a, b2Body* b, const float* f, int flags,
                      std::unique_ptr<b2Joint> j = nullptr)
    {
        if (!Handle() || !a || !b) return nullptr;
        const int ia = a->m_index, ib = b->m_index;
        int id = -1;
        if (gb_create_joints(m_h, 0, 1, &type, &ia, &ib, f, &flags, &id) != GB_OK) return nullptr;
        if (!j) j.reset(new b2Joint());
        j->m_world = this;
        j->m_index = id;
        j->m_a = a;
        j->m_b = b;
        j->m_slot = m_joints.size();
        m_joints.push_back(std::move(j));
        return m_joints.back().get();
    }
    gb_world* Handle()
    {
        if (!m_h) {
            m_def.gravity_x = m_gravity.x;
            m_def.gravity_y = m_gravity.y;
            if (gb_world_create(1, &m_def, &m_h) != GB_OK) m_h = nullptr;
            // the broadphase tree's history, for GetTreeHeight, GetTreeBalance and GetTreeQuality
            if (m_h) gb_world_track_tree(m_h, 1);
            if (m_h && !m_autoClear) gb_world_set_settings(m_h, 0, &m_def, 0);
        }
        return m_h;
    }
    void ApplySettings()
    {
        m_def.gravity_x = m_gravity.x;
        m_def.gravity_y = m_gravity.y;
        if (m_h) gb_world_set_settings(m_h, 0, &m_def, m_autoClear ? 1 : 0);
    }
    void ReadContacts()
    {
        int n = 0;
        std::vector<int> ints(8);
        std::vector<float> flts(12);
        if (gb_get_contacts(m_h, 0, ints.data(), flts.data(), 0, &n) != GB_OK && n == 0) n = 0;
        ints.assign(8 * (size_t)(n > 0 ? n : 1), 0);
        flts.assign(12 * (size_t)(n > 0 ? n : 1), 0.0f);
        if (n > 0) gb_get_contacts(m_h, 0, ints.data(), flts.data(), n, &n);
        m_contacts.clear();
        for (int i = 0; i < n; ++i) {
            std::unique_ptr<b2Contact> c(new b2Contact());
            const int* I = &ints[8 * (size_t)i];
            const float* F = &flts[12 * (size_t)i];
            c->m_a = m_fixtureOfId[I[0]].first;
            c->m_b = m_fixtureOfId[I[1]].first;
            c->m_childA = m_fixtureOfId[I[0]].second;
            c->m_childB = m_fixtureOfId[I[1]].second;
            c->m_idA = I[0];
            c->m_idB = I[1];
            c->m_flags = I[2];
            b2Manifold& m = c->m_manifold;
            m.pointCount = I[3];
            m.type = (b2Manifold::Type)I[4];
            m.localNormal = b2Vec2(F[0], F[1]);
            m.localPoint = b2Vec2(F[2], F[3]);
            for (int p = 0; p < 2; ++p) {
                m.points[p].localPoint = b2Vec2(F[4 + 4 * p], F[5 + 4 * p]);
                m.points[p].normalImpulse = F[6 + 4 * p];
                m.points[p].tangentImpulse = F[7 + 4 * p];
                m.points[p].id = (uint32_t)I[5 + p];
            }
            m_contacts.push_back(std::move(c));
        }
        // b2Contact::GetNext: the world's list order (newest first)
        for (size_t k = 0; k < m_contacts.size(); ++k)
            m_contacts[k]->m_next = k + 1 < m_contacts.size() ? m_contacts[k + 1].get() : nullptr;
    }
    // Makes the recorded listener calls from index `first` on, with the contacts as they are now and
    // as they were before (m_contacts); returns the number of calls recorded so far.
    int Report(int first)
    {
        // b2World::IsLocked inside the listener's calls, as during the reference's Step
        struct Lock {
            bool& flag;
            explicit Lock(bool& f) : flag(f) { flag = true; }
            ~Lock() { flag = false; }
        } lock(m_locked);
        std::vector<std::unique_ptr<b2Contact>> old = std::move(m_contacts);
        ReadContacts();
        std::map<std::pair<int, int>, b2Contact*> now, before;
        for (auto& c : m_contacts) now[{c->m_idA, c->m_idB}] = c.get();
        for (auto& c : old) before[{c->m_idA, c->m_idB}] = c.get();
        int n = 0;
        gb_world_read_events(m_h, 0, nullptr, nullptr, 0, &n);
        std::vector<int> rec(4 * (size_t)(n > 0 ? n : 1));
        std::vector<float> imp(4 * (size_t)(n > 0 ? n : 1));
        if (n > 0) gb_world_read_events(m_h, 0, rec.data(), imp.data(), n, &n);
        const b2Manifold empty;
        for (int i = first; i < n; ++i) {
            const std::pair<int, int> key{rec[4 * i + 1], rec[4 * i + 2]};
            auto itNow = now.find(key);
            auto itOld = before.find(key);
            b2Contact* c = itNow != now.end() ? itNow->second : (itOld != before.end() ? itOld->second : nullptr);
            if (!c) continue;
            switch (rec[4 * i]) {
            case 0: m_listener->BeginContact(c); break;
            case 1: m_listener->EndContact(itOld != before.end() && itNow == now.end() ? itOld->second : c); break;
            case 2: m_listener->PreSolve(c, itOld != before.end() ? &itOld->second->m_manifold : &empty); break;
            default: {
                b2ContactImpulse ci;
                ci.count = rec[4 * i + 3];
                ci.normalImpulses[0] = imp[4 * i]; ci.normalImpulses[1] = imp[4 * i + 1];
                ci.tangentImpulses[0] = imp[4 * i + 2]; ci.tangentImpulses[1] = imp[4 * i + 3];
                m_listener->PostSolve(c, &ci);
            }
            }
        }
        // kept alive: a listener may hold the pointers until the next Step
        if (first == 0) m_old.clear();
        for (auto& c : old) m_old.push_back(std::move(c));
        return n;
    }

    b2Vec2 m_gravity;
    gb_world_def m_def{0.0f, 0.0f, 1, 1, 1, 0};
    bool m_autoClear = true;
    gb_world* m_h = nullptr;
    b2ContactListener* m_listener = nullptr;
    b2DestructionListener* m_destruction = nullptr;
    b2ContactFilter* m_filter = nullptr;
    b2Profile m_profile;
    std::vector<std::unique_ptr<b2Body>> m_bodies;
    std::vector<std::unique_ptr<b2Fixture>> m_fixtures;
    std::vector<std::pair<b2Fixture*, int>> m_fixtureOfId;  // device fixture id -> fixture, chain child
    std::vector<std::unique_ptr<b2Joint>> m_joints;
    std::vector<std::unique_ptr<b2Contact>> m_contacts, m_old;
    bool m_eventsOn = false;
    bool m_locked = false;
    bool m_contactsStale = true;  // the contact list must be read again (a step or a change since)
    std::vector<b2Contact*> m_contactView;
    std::vector<float> m_state;
    bool m_stale = true;
};

inline b2Fixture* b2Body::CreateFixture(const b2FixtureDef* def) { return m_world->AddFixture(this, def); }
inline void b2Body::DestroyFixture(b2Fixture* fixture)
{
    if (fixture && fixture->m_body == this) m_world->DestroyFixture(fixture);
}
inline b2Body* b2Body::GetNext() const { return m_world->PreviousAlive((size_t)m_index); }
inline b2Fixture* b2Body::GetFixtureList() const { return m_world->FixtureListOf(this); }
inline b2ContactEdge* b2Body::GetContactList()
{
    m_contactEdges.clear();
    for (b2Contact* c : m_world->Contacts()) {
        b2Body* a = c->GetFixtureA()->GetBody();
        b2Body* b = c->GetFixtureB()->GetBody();
        if (a != this && b != this) continue;
        b2ContactEdge e;
        e.other = a == this ? b : a;
        e.contact = c;
        m_contactEdges.push_back(e);
    }
    for (size_t i = 0; i < m_contactEdges.size(); ++i) {
        m_contactEdges[i].prev = i > 0 ? &m_contactEdges[i - 1] : nullptr;
        m_contactEdges[i].next = i + 1 < m_contactEdges.size() ? &m_contactEdges[i + 1] : nullptr;
    }
    return m_contactEdges.empty() ? nullptr : &m_contactEdges[0];
}
inline b2JointEdge* b2Body::GetJointList()
{
    m_jointEdges.clear();
    for (b2Joint* j = m_world->GetJointList(); j; j = j->GetNext()) {
        if (j->GetBodyA() != this && j->GetBodyB() != this) continue;
        b2JointEdge e;
        e.other = j->GetBodyA() == this ? j->GetBodyB() : j->GetBodyA();
        e.joint = j;
        m_jointEdges.push_back(e);
    }
    for (size_t i = 0; i < m_jointEdges.size(); ++i) {
        m_jointEdges[i].prev = i > 0 ? &m_jointEdges[i - 1] : nullptr;
        m_jointEdges[i].next = i + 1 < m_jointEdges.size() ? &m_jointEdges[i + 1] : nullptr;
    }
    return m_jointEdges.empty() ? nullptr : &m_jointEdges[0];
}
inline b2Fixture* b2Fixture::GetNext() const { return m_body->GetWorld()->PreviousFixture(m_slot, m_body); }
inline b2Joint* b2Joint::GetNext() const { return m_world->PreviousJoint(m_slot); }
inline void b2Contact::GetWorldManifold(b2WorldManifold* worldManifold) const
{
    worldManifold->Initialize(&m_manifold, m_a->GetBody()->GetTransform(), m_a->GetRadius(),
                              m_b->GetBody()->GetTransform(), m_b->GetRadius());
}
inline const float* b2Body::State() const { return m_world->BodyState(m_index); }
inline void b2Body::SetTransform(const b2Vec2& p, float angle) { m_world->Edit(m_index, GB_EDIT_SET_TRANSFORM, p.x, p.y, angle, 0.0f, true); }
inline void b2Body::SetLinearVelocity(const b2Vec2& v) { m_world->Edit(m_index, GB_EDIT_SET_LINEAR_VELOCITY, v.x, v.y, 0.0f, 0.0f, true); }
inline void b2Body::SetAngularVelocity(float w) { m_world->Edit(m_index, GB_EDIT_SET_ANGULAR_VELOCITY, w, 0.0f, 0.0f, 0.0f, true); }
inline void b2Body::SetAwake(bool flag) { m_world->Edit(m_index, GB_EDIT_SET_AWAKE, flag ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f, true); }
inline void b2Body::ApplyForce(const b2Vec2& f, const b2Vec2& p, bool wake) { m_world->Edit(m_index, GB_EDIT_APPLY_FORCE, f.x, f.y, p.x, p.y, wake); }
inline void b2Body::ApplyForceToCenter(const b2Vec2& f, bool wake) { m_world->Edit(m_index, GB_EDIT_APPLY_FORCE_TO_CENTER, f.x, f.y, 0.0f, 0.0f, wake); }
inline void b2Body::ApplyTorque(float torque, bool wake) { m_world->Edit(m_index, GB_EDIT_APPLY_TORQUE, torque, 0.0f, 0.0f, 0.0f, wake); }
inline void b2Body::ApplyLinearImpulse(const b2Vec2& i, const b2Vec2& p, bool wake) { m_world->Edit(m_index, GB_EDIT_APPLY_LINEAR_IMPULSE, i.x, i.y, p.x, p.y, wake); }
inline void b2Body::ApplyAngularImpulse(float impulse, bool wake) { m_world->Edit(m_index, GB_EDIT_APPLY_ANGULAR_IMPULSE, impulse, 0.0f, 0.0f, 0.0f, wake); }
inline void b2Body::SetType(b2BodyType type)
{
    if (m_world->SetBodyProperty(this, GB_BODY_TYPE, (float)type)) m_type = type;
}
inline void b2Body::SetActive(bool flag) { m_world->SetBodyProperty(this, GB_BODY_ACTIVE, flag ? 1.0f : 0.0f); }
inline void b2Body::SetFixedRotation(bool flag) { m_world->SetBodyProperty(this, GB_BODY_FIXED_ROTATION, flag ? 1.0f : 0.0f); }
inline void b2Body::SetBullet(bool flag) { m_world->SetBodyProperty(this, GB_BODY_BULLET, flag ? 1.0f : 0.0f); }
inline void b2Body::SetSleepingAllowed(bool flag) { m_world->SetBodyProperty(this, GB_BODY_SLEEPING_ALLOWED, flag ? 1.0f : 0.0f); }
inline void b2Body::SetLinearDamping(float d) { m_world->SetBodyProperty(this, GB_BODY_LINEAR_DAMPING, d); }
inline void b2Body::SetAngularDamping(float d) { m_world->SetBodyProperty(this, GB_BODY_ANGULAR_DAMPING, d); }
inline void b2Body::SetGravityScale(float scale) { m_world->SetBodyProperty(this, GB_BODY_GRAVITY_SCALE, scale); }
inline bool b2Joint::Set(int prop, float v0, float v1) { return m_world->SetJointProperty(this, prop, v0, v1); }
inline b2Vec2 b2Joint::GetReactionForce(float inv_dt) const
{
    float out[3];
    m_world->JointReaction(m_index, inv_dt, out);
    return b2Vec2(out[0], out[1]);
}
inline float b2Joint::GetReactionTorque(float inv_dt) const
{
    float out[3];
    m_world->JointReaction(m_index, inv_dt, out);
    return out[2];
}
inline bool b2Fixture::TestPoint(const b2Vec2& p) const
{
    const float in[8] = {p.x, p.y, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    float out[4];
    return m_body->GetWorld()->FixtureQuery(m_index, 0, in, out) && out[0] != 0.0f;
}
inline bool b2Fixture::RayCast(b2RayCastOutput* output, const b2RayCastInput& input, int childIndex) const
{
    const float in[8] = {input.p1.x, input.p1.y, input.p2.x, input.p2.y, input.maxFraction, 0.0f, 0.0f, 0.0f};
    float out[4];
    if (!m_body->GetWorld()->FixtureQuery(m_index + childIndex, 1, in, out) || out[0] == 0.0f) return false;
    output->normal = b2Vec2(out[1], out[2]);
    output->fraction = out[3];
    return true;
}
inline void b2Fixture::GetMassData(b2MassData* md) const
{
    const float in[8] = {0};
    float out[4];
    m_body->GetWorld()->FixtureQuery(m_index, 3, in, out);
    md->mass = out[0];
    md->center = b2Vec2(out[1], out[2]);
    md->I = out[3];
}
inline const b2AABB b2Fixture::GetAABB(int childIndex) const
{
    const float in[8] = {0};
    float out[4];
    m_body->GetWorld()->FixtureQuery(m_index + childIndex, 2, in, out);
    b2AABB a;
    a.lowerBound = b2Vec2(out[0], out[1]);
    a.upperBound = b2Vec2(out[2], out[3]);
    return a;
}
inline void b2Fixture::SetFriction(float friction)
{
    if (m_body->GetWorld()->SetFixtureProperty(this, GB_FIXTURE_FRICTION, friction)) m_def.friction = friction;
}
inline void b2Fixture::SetRestitution(float restitution)
{
    if (m_body->GetWorld()->SetFixtureProperty(this, GB_FIXTURE_RESTITUTION, restitution)) m_def.restitution = restitution;
}
inline void b2Fixture::SetDensity(float density)
{
    if (m_body->GetWorld()->SetFixtureProperty(this, GB_FIXTURE_DENSITY, density)) m_def.density = density;
}
inline void b2Fixture::SetSensor(bool sensor)
{
    if (m_body->GetWorld()->SetFixtureProperty(this, GB_FIXTURE_SENSOR, sensor ? 1.0f : 0.0f)) m_def.isSensor = sensor;
}
inline void b2Fixture::SetFilterData(const b2Filter& filter)
{
    if (m_body->GetWorld()->SetFixtureProperty(this, GB_FIXTURE_FILTER, (float)filter.categoryBits,
                                               (float)filter.maskBits, (float)filter.groupIndex))
        m_def.filter = filter;
}
inline void b2Body::SetMassData(const b2MassData* d)
{
    if (d) m_world->SetBodyProperty(this, GB_BODY_MASS_DATA, d->mass, d->center.x, d->center.y, d->I);
}
inline void b2Body::ResetMassData() { m_world->SetBodyProperty(this, GB_BODY_RESET_MASS_DATA, 0.0f); }
inline float b2Body::Info(int k) const
{
    float out[7] = {0};
    m_world->BodyInfo(m_index, out);
    return out[k];
}
inline int b2Body::InfoFlags() const
{
    float out[7] = {0};
    return m_world->BodyInfo(m_index, out);
}

inline void b2MouseJoint::SetTarget(const b2Vec2& target)
{
    m_target = target;
    m_world->Edit(m_index, GB_EDIT_MOUSE_TARGET, target.x, target.y, 0.0f, 0.0f, true);
}

inline void b2RevoluteJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor)
{
    bodyA = bA;
    bodyB = bB;
    localAnchorA = bA->GetLocalPoint(anchor);
    localAnchorB = bB->GetLocalPoint(anchor);
    referenceAngle = bB->GetAngle() - bA->GetAngle();
}
inline void b2DistanceJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchorA, const b2Vec2& anchorB)
{
    bodyA = bA;
    bodyB = bB;
    localAnchorA = bA->GetLocalPoint(anchorA);
    localAnchorB = bB->GetLocalPoint(anchorB);
    const float dx = anchorB.x - anchorA.x, dy = anchorB.y - anchorA.y;
    length = std::sqrt(dx * dx + dy * dy);
}
inline void b2WeldJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor)
{
    bodyA = bA;
    bodyB = bB;
    localAnchorA = bA->GetLocalPoint(anchor);
    localAnchorB = bB->GetLocalPoint(anchor);
    referenceAngle = bB->GetAngle() - bA->GetAngle();
}
inline void b2WheelJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor, const b2Vec2& axis)
{
    bodyA = bA;
    bodyB = bB;
    localAnchorA = bA->GetLocalPoint(anchor);
    localAnchorB = bB->GetLocalPoint(anchor);
    localAxisA = bA->GetLocalVector(axis);
}
inline void b2FrictionJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor)
{
    bodyA = bA;
    bodyB = bB;
    localAnchorA = bA->GetLocalPoint(anchor);
    localAnchorB = bB->GetLocalPoint(anchor);
}
inline void b2MotorJointDef::Initialize(b2Body* bA, b2Body* bB)
{
    bodyA = bA;
    bodyB = bB;
    linearOffset = bA->GetLocalPoint(bB->GetPosition());
    angularOffset = bB->GetAngle() - bA->GetAngle();
}
inline void b2PrismaticJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& anchor, const b2Vec2& axis)
{
    bodyA = bA;
    bodyB = bB;
    localAnchorA = bA->GetLocalPoint(anchor);
    localAnchorB = bB->GetLocalPoint(anchor);
    localAxisA = bA->GetLocalVector(axis);
    referenceAngle = bB->GetAngle() - bA->GetAngle();
}
inline void b2PulleyJointDef::Initialize(b2Body* bA, b2Body* bB, const b2Vec2& groundA, const b2Vec2& groundB,
                                         const b2Vec2& anchorA, const b2Vec2& anchorB, float r)
{
    // the anchors in each body's frame (the transpose of its rotation applied to anchor - position)
    auto local = [](const b2Transform& t, const b2Vec2& p) {
        const float dx = p.x - t.p.x, dy = p.y - t.p.y;
        return b2Vec2(t.q.c * dx + t.q.s * dy, -t.q.s * dx + t.q.c * dy);
    };
    bodyA = bA;
    bodyB = bB;
    groundAnchorA = groundA;
    groundAnchorB = groundB;
    localAnchorA = local(bA->GetTransform(), anchorA);
    localAnchorB = local(bB->GetTransform(), anchorB);
    const float ax = anchorA.x - groundA.x, ay = anchorA.y - groundA.y;
    const float bx = anchorB.x - groundB.x, by = anchorB.y - groundB.y;
    lengthA = std::sqrt(ax * ax + ay * ay);
    lengthB = std::sqrt(bx * bx + by * by);
    ratio = r;
}

} // namespace box2d
