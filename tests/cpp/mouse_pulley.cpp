// A pulley joint made with b2PulleyJointDef::Initialize and a box dragged by a mouse joint whose
// target moves every step through static_cast<b2MouseJoint*>(...)->SetTarget, as user code of the
// reference writes it: a ground box at (0, -10), a fixture-less static anchor, pulley boxes at
// (-3, 5) and (3, 4) hanging from (-3, 10) and (3, 10) (ratio 1.2), and a 1 x 1 m box at (0, 3)
// held at (0.25, 3.25). 120 steps of 1/60 s at 8/3 iterations; prints step and the three dynamic
// bodies' positions and angles as hex floats.
#include <cstdio>

#include "box2d_gb300.hpp"

using namespace box2d;

static b2Body* Box(b2World& world, float x, float y, float hx, float hy, float density)
{
    b2BodyDef bd;
    bd.type = b2_dynamicBody;
    bd.position.Set(x, y);
    b2Body* b = world.CreateBody(&bd);
    b2PolygonShape shape;
    shape.SetAsBox(hx, hy);
    b->CreateFixture(&shape, density);
    return b;
}

int main()
{
    b2World world(b2Vec2(0.0f, -10.0f));
    b2BodyDef groundDef;
    groundDef.position.Set(0.0f, -10.0f);
    b2Body* ground = world.CreateBody(&groundDef);
    b2PolygonShape groundBox;
    groundBox.SetAsBox(50.0f, 10.0f);
    ground->CreateFixture(&groundBox, 0.0f);
    b2BodyDef anchorDef;
    b2Body* anchor = world.CreateBody(&anchorDef);

    b2Body* a = Box(world, -3.0f, 5.0f, 0.5f, 1.0f, 1.0f);
    b2Body* b = Box(world, 3.0f, 4.0f, 0.5f, 1.0f, 1.0f);
    b2PulleyJointDef pd;
    pd.Initialize(a, b, b2Vec2(-3.0f, 10.0f), b2Vec2(3.0f, 10.0f), b2Vec2(-3.0f, 6.0f), b2Vec2(3.0f, 5.0f), 1.2f);
    world.CreateJoint(&pd);

    b2Body* dragged = Box(world, 0.0f, 3.0f, 0.5f, 0.5f, 1.0f);
    b2MouseJointDef md;
    md.bodyA = anchor;
    md.bodyB = dragged;
    md.target.Set(0.25f, 3.25f);
    md.maxForce = 200.0f;
    b2MouseJoint* mouse = static_cast<b2MouseJoint*>(world.CreateJoint(&md));

    b2Body* dyn[3] = {a, b, dragged};
    for (int i = 0; i < 120; ++i) {
        if (i >= 10 && i < 70) mouse->SetTarget(b2Vec2(0.25f + 0.125f * (float)(i - 10), 3.25f));
        world.Step(1.0f / 60.0f, 8, 3);
        std::printf("%d", i);
        for (b2Body* d : dyn) {
            const b2Vec2 p = d->GetPosition();
            std::printf(" %a %a %a", p.x, p.y, d->GetAngle());
        }
        std::printf("\n");
    }
    return 0;
}
