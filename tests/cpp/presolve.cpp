// A PreSolve listener that changes contacts, through the C++ mirror of b2World: a 3-row box pyramid
// with 4 boxes dropped on it; contacts between two "ghost" boxes are disabled (SetEnabled(false)),
// between two "ice" boxes lose their friction, between two "bouncy" boxes get restitution 0.9. Prints
// every body's position, angle and velocity as hex floats after 120 steps.
#include <cstdio>
#include <vector>

#include "box2d_gb300.hpp"

using namespace box2d;

static int Bits(int fixture)
{
    // fixture 0 is the ground; boxes 1..13
    if (fixture == 0) return 0;
    return (fixture % 3 == 0 ? 1 : 0) | (fixture % 4 == 0 ? 2 : 0) | (fixture % 5 == 0 ? 4 : 0);
}

struct Rule : b2ContactListener {
    int changed = 0;
    void PreSolve(b2Contact* contact, const b2Manifold*) override
    {
        const int both = Bits(contact->GetFixtureA()->GetIndex()) & Bits(contact->GetFixtureB()->GetIndex());
        if (both & 1) contact->SetEnabled(false);
        if (both & 2) contact->SetFriction(0.0f);
        if (both & 4) contact->SetRestitution(0.9f);
        changed += both != 0;
    }
};

int main()
{
    b2World world(b2Vec2(0.0f, -10.0f));
    Rule rule;
    world.SetContactListener(&rule);
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
    std::printf("changed %d\n", rule.changed);
    return 0;
}
