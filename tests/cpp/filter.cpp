// A user b2ContactFilter through the C++ mirror of b2World: a 3-row box pyramid with 4 boxes dropped on
// it; the ground's pairs keep the default filter, two boxes collide unless the sum of their fixture
// indices is a multiple of 5. Prints every body's position, angle and velocity as hex floats after
// 120 steps.
#include <cstdio>
#include <vector>

#include "box2d_gb300.hpp"

using namespace box2d;

struct SumFilter : b2ContactFilter {
    int asked = 0;
    bool ShouldCollide(b2Fixture* a, b2Fixture* b) override
    {
        ++asked;
        if (a->GetIndex() == 0 || b->GetIndex() == 0) return b2ContactFilter::ShouldCollide(a, b);
        return (a->GetIndex() + b->GetIndex()) % 5 != 0;
    }
};

int main()
{
    b2World world(b2Vec2(0.0f, -10.0f));
    SumFilter filter;
    world.SetContactFilter(&filter);
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
    auto box = [&](float x, float y) {
        b2BodyDef bd;
        bd.type = b2_dynamicBody;
        bd.position.Set(x, y);
        b2Body* b = world.CreateBody(&bd);
        b2PolygonShape shape;
        shape.SetAsBox(0.5f, 0.5f);
        b2FixtureDef fd;
        fd.shape = &shape;
        fd.density = 5.0f;
        fd.friction = 0.6f;
        b->CreateFixture(&fd);
        bodies.push_back(b);
    };
    for (int r = 0; r < 3; ++r)
        for (int j = 0; j < 4 - r; ++j) box((float)(-1.875 + r * 0.625 + j * 1.25), (float)(0.5 + r * 1.0));
    for (int k = 0; k < 4; ++k) box(-1.5f + 1.0f * k, 5.0f + 1.5f * k);
    for (int i = 0; i < 120; ++i) world.Step(1.0f / 60.0f, 8, 3);
    for (b2Body* b : bodies) {
        const b2Vec2 p = b->GetPosition(), v = b->GetLinearVelocity();
        std::printf("body %d %a %a %a %a %a %a\n", b->GetIndex(), p.x, p.y, b->GetAngle(), v.x, v.y,
                    b->GetAngularVelocity());
    }
    std::printf("asked %d\n", filter.asked);
    return 0;
}
