// Destruction, world queries and getters through the C++ mirror of b2World (include/box2d_gb300.hpp):
// a box pyramid, a pendulum on a revolute joint and a two-fixture body; bodies, a fixture and (with its
// anchor body) the joint are destroyed between steps and a body is created after them. Prints the
// listener calls, the body states as hex floats, the body list, the proxy count, query and ray-cast
// callback results, the first contact's world manifold, the broadphase tree's height, balance and
// quality, and whether the profile was filled.
#include <cstdio>
#include <vector>

#include "box2d_gb300.hpp"

using namespace box2d;

struct Listener : b2ContactListener, b2DestructionListener {
    int ends = 0;
    std::vector<int> goodbyes;  // kind (0 joint, 1 fixture), index
    void EndContact(b2Contact*) override { ++ends; }
    void SayGoodbye(b2Joint* j) override { goodbyes.push_back(0); goodbyes.push_back(j->GetIndex()); }
    void SayGoodbye(b2Fixture* f) override { goodbyes.push_back(1); goodbyes.push_back(f->GetIndex()); }
};

struct AllQuery : b2QueryCallback {
    std::vector<int> ids;
    int stopAfter = -1;
    bool ReportFixture(b2Fixture* f) override
    {
        ids.push_back(f->GetIndex());
        return stopAfter < 0 || (int)ids.size() < stopAfter;
    }
};

struct Closest : b2RayCastCallback {
    int id = -1;
    float fraction = 1.0f;
    b2Vec2 point, normal;
    float ReportFixture(b2Fixture* f, const b2Vec2& p, const b2Vec2& n, float fr) override
    {
        id = f->GetIndex();
        fraction = fr;
        point = p;
        normal = n;
        return fr;
    }
};

struct Every : b2RayCastCallback {
    int hits = 0;
    float ReportFixture(b2Fixture*, const b2Vec2&, const b2Vec2&, float) override
    {
        ++hits;
        return 1.0f;
    }
};

static void Step(b2World& w, int n)
{
    for (int i = 0; i < n; ++i) w.Step(1.0f / 60.0f, 8, 3);
}

int main()
{
    b2World world(b2Vec2(0.0f, -10.0f));
    Listener listener;
    world.SetContactListener(&listener);
    world.SetDestructionListener(&listener);
    std::vector<b2Body*> bodies;

    b2BodyDef gd;
    b2Body* ground = world.CreateBody(&gd);
    b2EdgeShape edge;
    edge.Set(b2Vec2(-20.0f, 0.0f), b2Vec2(20.0f, 0.0f));
    b2FixtureDef ef;
    ef.shape = &edge;
    ef.friction = 0.6f;
    ground->CreateFixture(&ef);
    bodies.push_back(ground);
    for (int r = 0; r < 3; ++r)
        for (int j = 0; j < 4 - r; ++j) {
            b2BodyDef bd;
            bd.type = b2_dynamicBody;
            bd.position.Set((float)(-1.875 + r * 0.625 + j * 1.25), (float)(0.5 + r * 1.0));
            b2Body* b = world.CreateBody(&bd);
            b2PolygonShape box;
            box.SetAsBox(0.5f, 0.5f);
            b2FixtureDef fd;
            fd.shape = &box;
            fd.density = 5.0f;
            fd.friction = 0.6f;
            b->CreateFixture(&fd);
            bodies.push_back(b);
        }
    b2BodyDef ad;
    ad.position.Set(6.0f, 6.0f);
    b2Body* anchor = world.CreateBody(&ad);
    b2CircleShape small;
    small.m_radius = 0.25f;
    anchor->CreateFixture(&small, 0.0f);
    bodies.push_back(anchor);
    b2BodyDef pd;
    pd.type = b2_dynamicBody;
    pd.position.Set(8.0f, 6.0f);
    b2Body* bob = world.CreateBody(&pd);
    b2CircleShape ball;
    ball.m_radius = 0.5f;
    b2Fixture* bobFixture = bob->CreateFixture(&ball, 1.0f);
    bodies.push_back(bob);
    b2RevoluteJointDef jd;
    jd.bodyA = anchor;
    jd.bodyB = bob;
    jd.localAnchorA.Set(0.0f, 0.0f);
    jd.localAnchorB.Set(-2.0f, 0.0f);
    world.CreateJoint(&jd);
    b2BodyDef td;
    td.type = b2_dynamicBody;
    td.position.Set(-6.0f, 3.0f);
    b2Body* two = world.CreateBody(&td);
    b2PolygonShape plank;
    plank.SetAsBox(0.5f, 0.25f);
    two->CreateFixture(&plank, 1.0f);
    b2CircleShape knob;
    knob.m_p.Set(0.5f, 0.0f);
    knob.m_radius = 0.25f;
    b2Fixture* knobFixture = two->CreateFixture(&knob, 2.0f);
    bodies.push_back(two);

    Step(world, 40);
    world.DestroyBody(bodies[5]);
    two->DestroyFixture(knobFixture);
    std::printf("ends_after_first %d\n", listener.ends);
    Step(world, 20);
    world.DestroyBody(anchor);
    b2BodyDef nd;
    nd.type = b2_dynamicBody;
    nd.position.Set(0.0f, 8.0f);
    b2Body* late = world.CreateBody(&nd);
    b2PolygonShape lbox;
    lbox.SetAsBox(0.5f, 0.5f);
    late->CreateFixture(&lbox, 1.0f);
    bodies.push_back(late);
    Step(world, 40);

    std::printf("goodbyes");
    for (int g : listener.goodbyes) std::printf(" %d", g);
    std::printf("\nends %d bodies %d joints %d proxies %d\n", listener.ends, world.GetBodyCount(),
                world.GetJointCount(), world.GetProxyCount());
    std::printf("list");
    for (b2Body* b = world.GetBodyList(); b; b = b->GetNext()) std::printf(" %d", b->GetIndex());
    std::printf("\n");
    for (b2Body* b : bodies) {
        const b2Vec2 p = b->GetPosition(), v = b->GetLinearVelocity();
        std::printf("body %d %a %a %a %a %a %a\n", b->GetIndex(), p.x, p.y, b->GetAngle(), v.x, v.y,
                    b->GetAngularVelocity());
    }
    b2AABB box;
    box.lowerBound.Set(-3.0f, -1.0f);
    box.upperBound.Set(3.0f, 2.0f);
    AllQuery all;
    world.QueryAABB(&all, box);
    AllQuery two2;
    two2.stopAfter = 2;
    world.QueryAABB(&two2, box);
    std::printf("query");
    for (int id : all.ids) std::printf(" %d", id);
    std::printf("\nquery_stop");
    for (int id : two2.ids) std::printf(" %d", id);
    std::printf("\n");
    Closest closest;
    world.RayCast(&closest, b2Vec2(-10.0f, 0.75f), b2Vec2(10.0f, 0.25f));
    Every every;
    world.RayCast(&every, b2Vec2(-10.0f, 0.75f), b2Vec2(10.0f, 0.25f));
    std::printf("ray %d %a %a %a %a %a hits %d\n", closest.id, closest.fraction, closest.point.x, closest.point.y,
                closest.normal.x, closest.normal.y, every.hits);
    // the world manifold of the first contact in the list that has points (a new contact has none)
    std::vector<b2Contact*> contacts;  // the world's list, walked as the reference's
    for (b2Contact* c = world.GetContactList(); c; c = c->GetNext()) contacts.push_back(c);
    for (size_t k = 0; k < contacts.size(); ++k) {
        const b2Contact* c = contacts[k];
        if (c->GetManifold()->pointCount == 0) continue;
        b2WorldManifold wm;
        c->GetWorldManifold(&wm);
        std::printf("manifold %d %d %d %d %a %a %a %a %a %a %a %a\n", (int)k, c->GetFixtureA()->GetIndex(),
                    c->GetFixtureB()->GetIndex(), c->GetManifold()->pointCount, wm.normal.x, wm.normal.y,
                    wm.points[0].x, wm.points[0].y, wm.points[1].x, wm.points[1].y, wm.separations[0],
                    wm.separations[1]);
        break;
    }
    std::printf("tree %d %d %a\n", world.GetTreeHeight(), world.GetTreeBalance(), world.GetTreeQuality());
    // each body's contact edges (b2Body::GetContactList): how many, and the other bodies in order
    std::printf("edges");
    for (b2Body* b : bodies) {
        int n = 0;
        for (b2ContactEdge* e = b->GetContactList(); e; e = e->next) ++n;
        std::printf(" %d:%d", b->GetIndex(), n);
    }
    std::printf("\n");
    {
        const b2Vec2 c = bob->GetPosition();
        b2RayCastInput in;
        in.p1.Set(c.x - 2.0f, c.y + 0.1f);
        in.p2.Set(c.x + 2.0f, c.y - 0.1f);
        in.maxFraction = 1.0f;
        b2RayCastOutput out;
        const bool hit = bobFixture->RayCast(&out, in, 0);
        const b2AABB box = bobFixture->GetAABB(0);
        std::printf("fixq %d %d %a %a %a %a %a %a %a\n", bobFixture->TestPoint(c) ? 1 : 0, hit ? 1 : 0, out.normal.x,
                    out.normal.y, out.fraction, box.lowerBound.x, box.lowerBound.y, box.upperBound.x, box.upperBound.y);
    }
    const b2Profile& prof = world.GetProfile();
    std::printf("profile %d\n", prof.step > 0.0f && prof.solve > 0.0f ? 1 : 0);
    return 0;
}
