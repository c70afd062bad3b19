// The HelloWorld scene (a 100 x 20 m static ground box at (0, -10), a 2 x 2 m dynamic box of density
// 1 and friction 0.3 dropped from (0, 4)) driven through the C++ mirror's b2Body state changes
// between steps: an off-centre linear impulse, a teleport, a spin, a force at a point, a torque, and
// putting the body to sleep; 90 steps of 1/60 s at 8/3 iterations. Prints step, position, angle and
// awake flag as hex floats.
#include <cstdio>

#include "box2d_gb300.hpp"

using namespace box2d;

int main()
{
    b2World world(b2Vec2(0.0f, -10.0f));
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

    for (int i = 0; i < 90; ++i) {
        if (i == 10) body->ApplyLinearImpulse(b2Vec2(3.0f, 6.0f), b2Vec2(0.5f, 3.0f), true);
        if (i == 25) body->SetTransform(b2Vec2(-4.0f, 6.0f), 0.6f);
        if (i == 30) body->SetAngularVelocity(3.0f);
        if (i == 40) body->ApplyForce(b2Vec2(50.0f, 0.0f), b2Vec2(-4.0f, 1.0f), true);
        if (i == 41) body->ApplyTorque(-20.0f, true);
        if (i == 60) body->SetLinearVelocity(b2Vec2(1.0f, 0.0f));
        if (i == 75) body->SetAwake(false);
        world.Step(1.0f / 60.0f, 8, 3);
        const b2Vec2 p = body->GetPosition();
        std::printf("%d %a %a %a %d\n", i, p.x, p.y, body->GetAngle(), body->IsAwake() ? 1 : 0);
    }
    return 0;
}
