// b2Body property changes between steps through the C++ mirror of b2World (include/box2d_gb300.hpp):
// a box pyramid, a pendulum on a revolute joint and a two-fixture body; a loaded box turns static and
// back, an upper box is deactivated and activated again, and the pendulum, the two-fixture body and
// other boxes get gravity scale, damping, fixed rotation, bullet and sleeping changes, user mass data
// and a mass reset; box fixtures get friction, restitution, sensor and filter-group changes. Prints the EndContact count after the first changes and at the end, the body
// states as hex floats, the mass data, damping and flags of some bodies, and the pendulum bob's
// frame conversions.
#include <cstdio>
#include <vector>

#include "box2d_gb300.hpp"

using namespace box2d;

struct Listener : b2ContactListener {
    int ends = 0;
    void EndContact(b2Contact*) override { ++ends; }
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
    std::vector<b2Body*> bodies;
    std::vector<b2Fixture*> boxFixtures(1, nullptr);  // the boxes' fixtures, by body index

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
            boxFixtures.push_back(b->CreateFixture(&fd));
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
    bob->CreateFixture(&ball, 1.0f);
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
    two->CreateFixture(&knob, 2.0f);
    bodies.push_back(two);

    Step(world, 40);
    bodies[2]->SetType(b2_staticBody);
    bodies[8]->SetActive(false);
    bob->SetGravityScale(0.5f);
    bob->SetLinearDamping(0.5f);
    boxFixtures[4]->SetFriction(0.0f);
    boxFixtures[3]->SetRestitution(0.5f);
    boxFixtures[7]->SetSensor(true);
    b2Filter group;
    group.groupIndex = -3;
    boxFixtures[8]->SetFilterData(group);
    boxFixtures[9]->SetFilterData(group);
    std::printf("ends_after_first %d type %d\n", listener.ends, (int)bodies[2]->GetType());
    Step(world, 20);
    bodies[8]->SetActive(true);
    bodies[2]->SetType(b2_dynamicBody);
    boxFixtures[7]->SetSensor(false);
    boxFixtures[9]->Refilter();
    two->SetFixedRotation(true);
    bodies[9]->SetBullet(true);
    bodies[1]->SetSleepingAllowed(false);
    bob->SetAngularDamping(0.3f);
    b2MassData md;
    md.mass = 3.0f;
    md.center.Set(0.2f, -0.1f);
    md.I = 2.5f;
    bodies[5]->SetMassData(&md);
    Step(world, 20);
    bodies[6]->SetMassData(&md);
    bodies[6]->ResetMassData();
    Step(world, 20);

    std::printf("ends %d\n", listener.ends);
    for (int i : {1, 2, 5, 6, 9, 11, 12}) {
        b2Body* b = bodies[i];
        const b2Vec2 lc = b->GetLocalCenter();
        std::printf("info %d %a %a %a %a %a %a %a %d %d %d %d %d\n", i, b->GetMass(), b->GetInertia(), lc.x, lc.y,
                    b->GetLinearDamping(), b->GetAngularDamping(), b->GetGravityScale(), (int)b->GetType(),
                    b->IsBullet() ? 1 : 0, b->IsFixedRotation() ? 1 : 0, b->IsSleepingAllowed() ? 1 : 0,
                    b->IsActive() ? 1 : 0);
    }
    const b2Vec2 wp = bob->GetWorldPoint(b2Vec2(0.5f, 0.25f)), wv = bob->GetWorldVector(b2Vec2(0.5f, 0.25f));
    const b2Vec2 lp = bob->GetLocalPoint(b2Vec2(7.0f, 3.0f)), lv = bob->GetLocalVector(b2Vec2(7.0f, 3.0f));
    const b2Vec2 vw = bob->GetLinearVelocityFromWorldPoint(b2Vec2(7.0f, 3.0f));
    const b2Vec2 vl = bob->GetLinearVelocityFromLocalPoint(b2Vec2(0.5f, 0.25f));
    std::printf("frames %a %a %a %a %a %a %a %a %a %a %a %a\n", wp.x, wp.y, wv.x, wv.y, lp.x, lp.y, lv.x, lv.y, vw.x,
                vw.y, vl.x, vl.y);
    for (b2Body* b : bodies) {
        const b2Vec2 p = b->GetPosition(), v = b->GetLinearVelocity();
        std::printf("body %d %a %a %a %a %a %a\n", b->GetIndex(), p.x, p.y, b->GetAngle(), v.x, v.y,
                    b->GetAngularVelocity());
    }
    return 0;
}
