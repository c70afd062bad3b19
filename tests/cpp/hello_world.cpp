// The Box2D manual's HelloWorld through the C++ mirror of b2World (include/box2d_gb300.hpp): a 100 x
// 20 m static ground box at (0, -10), a 2 x 2 m dynamic box (density 1, friction 0.3) dropped from
// (0, 4), 60 steps of 1/60 s at 6/2 iterations. Prints step, position and angle as hex floats and
// the contact events a listener saw.
#include <cstdio>

#include "box2d_gb300.hpp"

using namespace box2d;

struct Counter : b2ContactListener {
    int begins = 0, ends = 0, presolves = 0, postsolves = 0;
    float lastNormalImpulse = 0.0f;
    void BeginContact(b2Contact*) override { ++begins; }
    void EndContact(b2Contact*) override { ++ends; }
    void PreSolve(b2Contact*, const b2Manifold*) override { ++presolves; }
    void PostSolve(b2Contact*, const b2ContactImpulse* impulse) override
    {
        ++postsolves;
        lastNormalImpulse = impulse->normalImpulses[0];
    }
};

int main()
{
    b2World world(b2Vec2(0.0f, -10.0f));
    Counter counter;
    world.SetContactListener(&counter);

    b2BodyDef groundBodyDef;
    groundBodyDef.position.Set(0.0f, -10.0f);
    b2Body* groundBody = world.CreateBody(&groundBodyDef);
    b2PolygonShape groundBox;
    groundBox.SetAsBox(50.0f, 10.0f);
    groundBody->CreateFixture(&groundBox, 0.0f);

    b2BodyDef bodyDef;
    bodyDef.type = b2_dynamicBody;
    bodyDef.position.Set(0.0f, 4.0f);
    b2Body* body = world.CreateBody(&bodyDef);
    b2PolygonShape dynamicBox;
    dynamicBox.SetAsBox(1.0f, 1.0f);
    b2FixtureDef fixtureDef;
    fixtureDef.shape = &dynamicBox;
    fixtureDef.density = 1.0f;
    fixtureDef.friction = 0.3f;
    body->CreateFixture(&fixtureDef);

    const float timeStep = 1.0f / 60.0f;
    for (int i = 0; i < 60; ++i) {
        world.Step(timeStep, 6, 2);
        const b2Vec2 p = body->GetPosition();
        std::printf("%d %a %a %a\n", i, p.x, p.y, body->GetAngle());
    }
    std::printf("contacts %d begin %d end %d awake %d presolve %d postsolve %d impulse %a\n", world.GetContactCount(),
                counter.begins, counter.ends, body->IsAwake() ? 1 : 0, counter.presolves, counter.postsolves,
                counter.lastNormalImpulse);
    return 0;
}
