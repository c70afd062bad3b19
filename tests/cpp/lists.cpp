// The b2World lists and user data of the C++ mirror without stepping: b2Body::GetFixtureList with
// b2Fixture::GetNext, b2World::GetJointList with b2Joint::GetNext (newest first, destroyed entries
// left out, as the reference's lists), and SetUserData / GetUserData of bodies, fixtures and joints.
// Prints each list as indices.
#include <cstdio>

#include "box2d_gb300.hpp"

using namespace box2d;

int main()
{
    b2World world(b2Vec2(0.0f, -10.0f));
    b2BodyDef gd;
    b2Body* ground = world.CreateBody(&gd);
    b2BodyDef bd;
    bd.type = b2_dynamicBody;
    bd.position.Set(0.0f, 2.0f);
    b2Body* body = world.CreateBody(&bd);
    b2PolygonShape box;
    box.SetAsBox(0.5f, 0.5f);
    b2CircleShape ball;
    ball.m_radius = 0.25f;
    b2Fixture* f0 = body->CreateFixture(&box, 1.0f);
    b2Fixture* f1 = body->CreateFixture(&ball, 1.0f);
    b2Fixture* f2 = body->CreateFixture(&box, 2.0f);
    ground->CreateFixture(&box, 0.0f);
    b2RevoluteJointDef rd;
    rd.bodyA = ground;
    rd.bodyB = body;
    b2Joint* j0 = world.CreateJoint(&rd);
    b2DistanceJointDef dd;
    dd.bodyA = ground;
    dd.bodyB = body;
    b2Joint* j1 = world.CreateJoint(&dd);
    b2Joint* j2 = world.CreateJoint(&rd);
    int tags[3] = {7, 8, 9};
    body->SetUserData(&tags[0]);
    f1->SetUserData(&tags[1]);
    j2->SetUserData(&tags[2]);

    std::printf("fixtures");
    for (b2Fixture* f = body->GetFixtureList(); f; f = f->GetNext()) std::printf(" %d", f->GetIndex());
    std::printf("\njoints");
    for (b2Joint* j = world.GetJointList(); j; j = j->GetNext()) std::printf(" %d", j->GetIndex());
    std::printf("\n");
    body->DestroyFixture(f1);
    world.DestroyJoint(j1);
    std::printf("fixtures_after");
    for (b2Fixture* f = body->GetFixtureList(); f; f = f->GetNext()) std::printf(" %d", f->GetIndex());
    std::printf("\njoints_after");
    for (b2Joint* j = world.GetJointList(); j; j = j->GetNext()) std::printf(" %d", j->GetIndex());
    std::printf("\nuser %d %d %d\n", *static_cast<int*>(body->GetUserData()), *static_cast<int*>(f1->GetUserData()),
                *static_cast<int*>(j2->GetUserData()));
    std::printf("body_joints");
    for (b2JointEdge* e = body->GetJointList(); e; e = e->next)
        std::printf(" %d:%d", e->joint->GetIndex(), e->other == ground ? 0 : 1);
    std::printf("\nground_contacts %d\n", ground->GetContactList() ? 1 : 0);
    std::printf("ground_fixtures");
    for (b2Fixture* f = ground->GetFixtureList(); f; f = f->GetNext()) std::printf(" %d", f->GetIndex());
    std::printf("\n");
    (void)f0;
    (void)f2;
    (void)j0;
    return 0;
}
