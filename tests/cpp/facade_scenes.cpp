// Host program written against the solver facade (include/avbdg_solver.hpp) the way host code
// drives the reference's avbd::Solver: fields assigned, bodies and joints constructed into the
// solver, step() called, Rigid fields read back. Prints the FNV-1a state digest of three scenes
// (bodies in list order: position, orientation, linear and angular velocity), the digest the
// reference's suite pins for them.
#include <cstdio>
#include <cstring>

#include "avbdg_solver.hpp"

using namespace avbdg;

static unsigned long long digest(const Solver &s) {
    unsigned long long h = 1469598103934665603ull;
    const auto mix = [&h](const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        for (size_t i = 0; i < n; i++) {
            h ^= c[i];
            h *= 1099511628211ull;
        }
    };
    for (const Rigid *b = s.bodies; b; b = b->next) {
        const float v[13] = {b->positionLin.x, b->positionLin.y, b->positionLin.z, b->positionAng.x, b->positionAng.y,
                             b->positionAng.z, b->positionAng.w, b->velocityLin.x, b->velocityLin.y,
                             b->velocityLin.z, b->velocityAng.x, b->velocityAng.y, b->velocityAng.z};
        mix(v, sizeof(v));
    }
    return h;
}

// Ground + 10 unit boxes stacked at z = 1.5 i + 1.
static void stack(Solver &s) {
    new Rigid(&s, float3{100, 100, 1}, ShapeType::Box, 0.0f, 0.5f, float3{0, 0, 0});
    for (int i = 0; i < 10; i++)
        new Rigid(&s, float3{1, 1, 1}, ShapeType::Box, 1.0f, 0.5f, float3{0, 0, float(i) * 1.5f + 1.0f});
}

int main() {
    {
        Solver s;
        stack(s);
        for (int i = 0; i < 300; i++)
            s.step();
        std::printf("stack %016llx\n", digest(s));
    }
    {
        Solver s;
        s.dt = 1.0f / 120.0f;
        stack(s);
        for (int i = 0; i < 300; i++)
            s.stepInterleaved(2, 3);
        std::printf("interleaved %016llx\n", digest(s));
    }
    {
        // 30-link chain (Joint 1000 / 250) beside 40 free boxes.
        Solver s;
        new Rigid(&s, float3{100, 100, 1}, ShapeType::Box, 0.0f, 0.5f, float3{0, 0, 0});
        Rigid *prev = nullptr;
        for (int i = 0; i < 30; i++) {
            Rigid *link = new Rigid(&s, float3{1, 1, 1}, ShapeType::Box, 1.0f, 0.5f, float3{0, 0, 20.0f - float(i) * 1.5f});
            if (prev)
                new Joint(&s, prev, link, float3{0, 0, -0.5f}, float3{0, 0, 0.5f}, 1000.0f, 250.0f);
            prev = link;
        }
        for (int i = 0; i < 40; i++)
            new Rigid(&s, float3{1, 1, 1}, ShapeType::Box, 1.0f, 0.5f,
                      float3{5.0f + float(i) * 1.2f, 0, 3.0f + float(i % 5)});
        for (int i = 0; i < 240; i++)
            s.step();
        std::printf("mixed %016llx manifolds %d colours %d\n", digest(s), s.manifoldCount(), s.colourGroups());
    }
    return 0;
}
