// Chain shapes through the C++ mirror as reference user code makes them: an open terrain chain with
// ghost vertices past both ends (b2ChainShape::CreateChain + SetPrevVertex/SetNextVertex) and a
// closed loop (CreateLoop) on a rotated static body, with boxes and circles dropped on them. 120
// steps of 1/60 s at 8/3 iterations. Prints each step's dynamic body positions as hex floats, then
// for every contact on a chain: the chain (0 terrain, 1 loop), the child index and the other
// fixture's body.
#include <cstdio>

#include "box2d_gb300.hpp"

using namespace box2d;

int main()
{
    b2World world(b2Vec2(0.0f, -10.0f));
    b2BodyDef groundDef;
    b2Body* ground = world.CreateBody(&groundDef);
    b2Vec2 terrain[9];
    for (int i = 0; i < 9; ++i) terrain[i].Set(-8.0f + 2.0f * (float)i, (i % 2) ? 0.5f : 0.0f);
    b2ChainShape open;
    open.CreateChain(terrain, 9);
    open.SetPrevVertex(b2Vec2(-10.0f, 1.0f));
    open.SetNextVertex(b2Vec2(10.0f, 1.0f));
    b2FixtureDef fd;
    fd.shape = &open;
    fd.friction = 0.6f;
    b2Fixture* terrainFixture = ground->CreateFixture(&fd);

    b2BodyDef boxDef;
    boxDef.position.Set(14.0f, 4.0f);
    boxDef.angle = 0.2f;
    b2Body* container = world.CreateBody(&boxDef);
    const b2Vec2 loop[4] = {b2Vec2(-3.0f, -2.0f), b2Vec2(3.0f, -2.0f), b2Vec2(3.0f, 2.0f), b2Vec2(-3.0f, 2.0f)};
    b2ChainShape closed;
    closed.CreateLoop(loop, 4);
    b2FixtureDef ld;
    ld.shape = &closed;
    ld.friction = 0.4f;
    b2Fixture* loopFixture = container->CreateFixture(&ld);

    b2Body* dyn[8];
    for (int i = 0; i < 8; ++i) {
        b2BodyDef bd;
        bd.type = b2_dynamicBody;
        bd.position.Set(i < 6 ? -7.0f + 2.5f * (float)i : 13.0f + 2.0f * (float)(i - 6), i < 6 ? 3.0f : 4.0f);
        bd.angle = 0.1f * (float)i;
        dyn[i] = world.CreateBody(&bd);
        b2FixtureDef f;
        f.density = 1.0f;
        f.friction = 0.4f;
        b2PolygonShape box;
        b2CircleShape circle;
        if (i % 2) {
            circle.m_radius = 0.4f;
            f.shape = &circle;
        } else {
            box.SetAsBox(0.4f, 0.3f);
            f.shape = &box;
        }
        dyn[i]->CreateFixture(&f);
    }

    for (int s = 0; s < 120; ++s) {
        world.Step(1.0f / 60.0f, 8, 3);
        std::printf("%d", s);
        for (b2Body* b : dyn) {
            const b2Vec2 p = b->GetPosition();
            std::printf(" %a %a", p.x, p.y);
        }
        std::printf("\n");
    }
    for (b2Contact* c = world.GetContactList(); c; c = c->GetNext()) {
        const b2Fixture* a = c->GetFixtureA();
        const int which = a == terrainFixture ? 0 : (a == loopFixture ? 1 : -1);
        if (which < 0) continue;
        std::printf("chain %d child %d body %d\n", which, c->GetChildIndexA(), c->GetFixtureB()->GetBody()->GetIndex());
    }
    return 0;
}
