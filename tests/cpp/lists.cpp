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
    std::printf("\nground_contacts %d %d\n", ground->GetContactList() ? 1 : 0, world.GetContactList() ? 1 : 0);
    std::printf("ground_fixtures");
    for (b2Fixture* f = ground->GetFixtureList(); f; f = f->GetNext()) std::printf(" %d", f->GetIndex());
    std::printf("\n");
    // joint definitions from world anchors (the defs' Initialize), between a turned body and another
    b2BodyDef ad;
    ad.type = b2_dynamicBody;
    ad.position.Set(1.25f, -0.5f);
    ad.angle = 0.7f;
    b2Body* a = world.CreateBody(&ad);
    b2BodyDef cd;
    cd.type = b2_dynamicBody;
    cd.position.Set(-2.0f, 3.5f);
    cd.angle = -1.3f;
    b2Body* c = world.CreateBody(&cd);
    const b2Vec2 anchor(0.3f, 1.1f), anchor2(-1.7f, 2.9f), axis(0.6f, 0.8f);
    for (b2Body* b : {a, c}) {
        const b2Transform t = b->GetTransform();
        std::printf("xf %a %a %a %a %a\n", t.p.x, t.p.y, t.q.s, t.q.c, b->GetAngle());
    }
    b2RevoluteJointDef rj;
    rj.Initialize(a, c, anchor);
    std::printf("rev %a %a %a %a %a\n", rj.localAnchorA.x, rj.localAnchorA.y, rj.localAnchorB.x, rj.localAnchorB.y,
                rj.referenceAngle);
    b2PrismaticJointDef pj;
    pj.Initialize(a, c, anchor, axis);
    std::printf("pri %a %a %a %a %a %a %a\n", pj.localAnchorA.x, pj.localAnchorA.y, pj.localAnchorB.x,
                pj.localAnchorB.y, pj.localAxisA.x, pj.localAxisA.y, pj.referenceAngle);
    b2WheelJointDef wj;
    wj.Initialize(a, c, anchor, axis);
    std::printf("whe %a %a %a %a %a %a\n", wj.localAnchorA.x, wj.localAnchorA.y, wj.localAnchorB.x, wj.localAnchorB.y,
                wj.localAxisA.x, wj.localAxisA.y);
    b2DistanceJointDef dj;
    dj.Initialize(a, c, anchor, anchor2);
    std::printf("dis %a %a %a %a %a\n", dj.localAnchorA.x, dj.localAnchorA.y, dj.localAnchorB.x, dj.localAnchorB.y,
                dj.length);
    b2MotorJointDef mj;
    mj.Initialize(a, c);
    std::printf("mot %a %a %a\n", mj.linearOffset.x, mj.linearOffset.y, mj.angularOffset);
    b2WeldJointDef weld;
    weld.Initialize(a, c, anchor);
    weld.userData = &tags[2];
    b2Joint* wjoint = world.CreateJoint(&weld);
    std::printf("weld_user %d\n", *static_cast<int*>(wjoint->GetUserData()));
    // b2PolygonShape as the reference holds it after Set and SetAsBox
    b2PolygonShape hull;
    const b2Vec2 pts[5] = {b2Vec2(0.0f, 0.0f), b2Vec2(1.5f, 0.2f), b2Vec2(0.7f, 1.1f), b2Vec2(0.6f, 0.5f),
                           b2Vec2(-0.4f, 0.9f)};
    hull.Set(pts, 5);
    b2PolygonShape turned;
    turned.SetAsBox(0.5f, 0.25f, b2Vec2(1.0f, -2.0f), 0.7f);
    for (const b2PolygonShape* s : {&hull, &turned}) {
        std::printf("poly %d %a %a", s->GetVertexCount(), s->m_centroid.x, s->m_centroid.y);
        for (int i = 0; i < s->m_count; ++i)
            std::printf(" %a %a %a %a", s->GetVertex(i).x, s->GetVertex(i).y, s->m_normals[i].x, s->m_normals[i].y);
        std::printf("\n");
    }
    (void)f0;
    (void)f2;
    (void)j0;
    return 0;
}
