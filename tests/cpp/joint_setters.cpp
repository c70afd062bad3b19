// Joint setters through the typed joints CreateJoint returns (static_cast<b2RevoluteJoint*>(...) and
// so on, as user code of the reference writes it): a box pendulum on a revolute joint, a box slider on
// a prismatic joint with limits, a car wheel on a wheel joint, two circles on a distance joint and a
// box held by a motor joint, all over an edge ground. 30 steps, then motors switched on and driven,
// limits set, springs, length and offsets changed; 60 more steps. Prints the revolute joint's getters,
// every joint's reaction force and torque, and every body's position, angle and velocities as hex
// floats.
#include <cstdio>

#include "box2d_gb300.hpp"

using namespace box2d;

static b2Body* Dynamic(b2World& world, float x, float y)
{
    b2BodyDef bd;
    bd.type = b2_dynamicBody;
    bd.position.Set(x, y);
    return world.CreateBody(&bd);
}

static void Box(b2Body* b, float hx, float hy, float density)
{
    b2PolygonShape shape;
    shape.SetAsBox(hx, hy);
    b->CreateFixture(&shape, density);
}

static void Circle(b2Body* b, float r, float density)
{
    b2CircleShape shape;
    shape.m_radius = r;
    b->CreateFixture(&shape, density);
}

int main()
{
    b2World world(b2Vec2(0.0f, -10.0f));
    std::vector<b2Body*> bodies;
    b2BodyDef gd;
    b2Body* ground = world.CreateBody(&gd);
    b2EdgeShape edge;
    edge.Set(b2Vec2(-20.0f, 0.0f), b2Vec2(20.0f, 0.0f));
    ground->CreateFixture(&edge, 0.0f);
    bodies.push_back(ground);

    b2Body* pendulum = Dynamic(world, 0.0f, 5.0f);
    Box(pendulum, 0.25f, 1.0f, 1.0f);
    bodies.push_back(pendulum);
    b2RevoluteJointDef rd;
    rd.bodyA = ground;
    rd.bodyB = pendulum;
    rd.localAnchorA.Set(0.0f, 6.0f);
    rd.localAnchorB.Set(0.0f, 1.0f);
    b2RevoluteJoint* rj = static_cast<b2RevoluteJoint*>(world.CreateJoint(&rd));

    b2Body* slider = Dynamic(world, 5.0f, 2.0f);
    Box(slider, 0.5f, 0.25f, 1.0f);
    bodies.push_back(slider);
    b2PrismaticJointDef pd;
    pd.bodyA = ground;
    pd.bodyB = slider;
    pd.localAnchorA.Set(5.0f, 2.0f);
    pd.localAxisA.Set(1.0f, 0.0f);
    pd.enableLimit = true;
    pd.lowerTranslation = -1.0f;
    pd.upperTranslation = 1.0f;
    b2PrismaticJoint* pj = static_cast<b2PrismaticJoint*>(world.CreateJoint(&pd));

    b2Body* chassis = Dynamic(world, -8.0f, 1.5f);
    Box(chassis, 1.0f, 0.25f, 1.0f);
    bodies.push_back(chassis);
    b2Body* wheel = Dynamic(world, -8.5f, 0.6f);
    Circle(wheel, 0.4f, 1.0f);
    bodies.push_back(wheel);
    b2WheelJointDef wd;
    wd.bodyA = chassis;
    wd.bodyB = wheel;
    wd.localAnchorA.Set(-0.5f, -0.9f);
    wd.localAxisA.Set(0.0f, 1.0f);
    wd.enableMotor = true;
    wd.maxMotorTorque = 20.0f;
    wd.frequencyHz = 4.0f;
    wd.dampingRatio = 0.7f;
    b2WheelJoint* wj = static_cast<b2WheelJoint*>(world.CreateJoint(&wd));

    b2Body* c1 = Dynamic(world, 10.0f, 6.0f);
    Circle(c1, 0.3f, 1.0f);
    bodies.push_back(c1);
    b2Body* c2 = Dynamic(world, 11.0f, 6.0f);
    Circle(c2, 0.3f, 1.0f);
    bodies.push_back(c2);
    b2DistanceJointDef dd;
    dd.bodyA = c1;
    dd.bodyB = c2;
    dd.length = 1.0f;
    b2DistanceJoint* dj = static_cast<b2DistanceJoint*>(world.CreateJoint(&dd));

    b2Body* held = Dynamic(world, -3.0f, 3.0f);
    Box(held, 0.3f, 0.3f, 1.0f);
    bodies.push_back(held);
    b2MotorJointDef md;
    md.bodyA = ground;
    md.bodyB = held;
    md.linearOffset.Set(-3.0f, 3.0f);
    md.maxForce = 100.0f;
    md.maxTorque = 10.0f;
    b2MotorJoint* mj = static_cast<b2MotorJoint*>(world.CreateJoint(&md));

    for (int i = 0; i < 30; ++i) world.Step(1.0f / 60.0f, 8, 3);
    rj->EnableMotor(true);
    rj->SetMotorSpeed(2.0f);
    rj->SetMaxMotorTorque(100.0f);
    rj->SetLimits(-0.5f, 0.5f);
    rj->EnableLimit(true);
    pj->EnableMotor(true);
    pj->SetMotorSpeed(-1.5f);
    pj->SetMaxMotorForce(50.0f);
    pj->SetLimits(-2.0f, 0.5f);
    wj->SetMotorSpeed(-15.0f);
    wj->SetMaxMotorTorque(60.0f);
    wj->SetSpringFrequencyHz(2.5f);
    wj->SetSpringDampingRatio(0.4f);
    dj->SetLength(1.6f);
    dj->SetFrequency(3.0f);
    dj->SetDampingRatio(0.2f);
    mj->SetLinearOffset(b2Vec2(-2.0f, 4.0f));
    mj->SetAngularOffset(0.5f);
    mj->SetMaxForce(300.0f);
    mj->SetMaxTorque(200.0f);
    mj->SetCorrectionFactor(0.5f);
    for (int i = 0; i < 60; ++i) world.Step(1.0f / 60.0f, 8, 3);

    std::printf("revolute %d %d %a %a %a %a\n", rj->IsMotorEnabled() ? 1 : 0, rj->IsLimitEnabled() ? 1 : 0,
                rj->GetMotorSpeed(), rj->GetMaxMotorTorque(), rj->GetLowerLimit(), rj->GetUpperLimit());
    const b2Joint* joints[5] = {rj, pj, wj, dj, mj};
    for (int k = 0; k < 5; ++k) {
        const b2Vec2 f = joints[k]->GetReactionForce(60.0f);
        std::printf("reaction %d %a %a %a\n", k, f.x, f.y, joints[k]->GetReactionTorque(60.0f));
    }
    for (size_t i = 0; i < bodies.size(); ++i) {
        const b2Vec2 p = bodies[i]->GetPosition(), v = bodies[i]->GetLinearVelocity();
        std::printf("body %d %a %a %a %a %a %a\n", (int)i, p.x, p.y, bodies[i]->GetAngle(), v.x, v.y,
                    bodies[i]->GetAngularVelocity());
    }
    return 0;
}
