// ref_physics.cpp -- TEST INFRASTRUCTURE ONLY (never linked into the product).
//
// Compiles the reference's own world::physicsCheck and world::physicsCheck_flood
// (source/engine/world.cpp:3330-3430), extracted unchanged by oracle/Makefile
// (target `ref`) into _ref/, with world::getTile (world.cpp:999-1002), so that the
// oracle's restatement and the device island kernels can be checked against them.
// This file supplies stand-ins for what the function hands its result to: an SDL
// surface that records its size and pixels, and a rigid body, texture, hitbox and
// world mesh that record nothing but the body's position.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

typedef float f32;
typedef uint32_t u32;
typedef uint8_t u8;

enum PhysicsType { AIR = 0, SOLID = 1, SAND = 2, SOUP = 3, GAS = 4, PASSABLE = 5, OBJECT = 5 };

struct Material {
    int id = 0;
    int physicsType = 0;
};
struct MaterialInstance {
    u32 id = 0;
    Material *mat = nullptr;
    u32 color = 0;
};

// the surface the cut region's colours go to
struct C_Surface {
    int w = 0, h = 0;
    std::vector<u32> px;
};
static const int SDL_PIXELFORMAT_ARGB8888 = 0;
static C_Surface *SDL_CreateRGBSurfaceWithFormat(int, int w, int h, int, int) {
    C_Surface *s = new C_Surface();
    s->w = w;
    s->h = h;
    s->px.assign((size_t)w * h, 0u);
    return s;
}
static u32 &ME_get_pixel(C_Surface *s, unsigned long long x, int y) { return s->px[(size_t)y * s->w + x]; }

// the rigid body side: records the surface and the body's position
struct Texture {
    C_Surface *sfc;
    explicit Texture(C_Surface *s) : sfc(s) {}
};
template <class T, class A>
static std::shared_ptr<T> create_ref(A a) {
    return std::make_shared<T>(a);
}
struct b2Vec2 {
    f32 x, y;
};
struct b2Filter {
    uint16_t categoryBits = 0, maskBits = 0;
};
struct b2Fixture {
    void SetFilterData(const b2Filter &) {}
};
struct b2Body {
    b2Fixture fix[1];
    b2Fixture *GetFixtureList() { return fix; }
    void SetLinearVelocity(b2Vec2) {}
};
struct b2PolygonShape {
    void SetAsBox(f32, f32) {}
};
static const int b2_dynamicBody = 2;
struct RigidBody {
    b2Body *body;
    f32 x, y;
    std::shared_ptr<Texture> tex;
};
struct MeshZone {
    int x = 0, y = 0, w = 0, h = 0;
};
static int fse_ref_rand() { return 0; }  // the body's initial velocity only
#define rand() fse_ref_rand()

static Material g_solid{1, SOLID};
static MaterialInstance Tiles_TEST_SOLID{1, &g_solid, 0xff0000};
static MaterialInstance Tiles_NOTHING{0, nullptr, 0};

struct world {
    int width = 0, height = 0;
    MaterialInstance *real_tiles = nullptr;
    bool *dirty = nullptr;
    std::vector<RigidBody *> rigidBodies;
    MeshZone lastMeshLoadZone;
    b2Body body;
    MaterialInstance getTile(int x, int y);
    RigidBody *makeRigidBody(int, f32 x, f32 y, f32, b2PolygonShape, f32, f32, std::shared_ptr<Texture> tex) {
        RigidBody *rb = new RigidBody{&body, x, y, tex};
        return rb;
    }
    void updateRigidBodyHitbox(RigidBody *) {}
    void updateWorldMesh() {}
    RigidBody *physicsCheck(int x, int y);
    void physicsCheck_flood(int x, int y, bool *visited, int *count, u32 *cols, int *minX, int *maxX, int *minY,
                            int *maxY);
};

#include "physics_gettile.inc"
#include "physics_check.inc"
#include "physics_flood.inc"

// One physicsCheck(x, y) on a grid of material types (0 AIR, 1 SOLID, ...) and
// colours; the cut cells become AIR (type 0) in `types`. Returns the surface's
// pixel count when a rigid body was made (its image in img, up to cap, origin in
// *ox, *oy, size in *w, *h), 0 when the region was removed without one or nothing
// happened (compare `types` before and after).
extern "C" long ref_physics_check(int W, int H, uint8_t *types, const uint32_t *cols, int x, int y, uint32_t *img,
                                  long cap, int *ox, int *oy, int *w, int *h) {
    std::vector<Material> mats(8);
    for (int i = 0; i < 8; i++) mats[i] = Material{i, i};
    std::vector<MaterialInstance> tiles((size_t)W * H);
    std::vector<char> dirty((size_t)W * H, 0);
    Material air{0, AIR};
    Tiles_NOTHING.mat = &air;
    for (size_t i = 0; i < tiles.size(); i++) tiles[i] = MaterialInstance{types[i], &mats[types[i] & 7], cols[i]};
    world wd;
    wd.width = W;
    wd.height = H;
    wd.real_tiles = tiles.data();
    wd.dirty = reinterpret_cast<bool *>(dirty.data());
    RigidBody *rb = wd.physicsCheck(x, y);
    for (size_t i = 0; i < tiles.size(); i++) types[i] = (uint8_t)tiles[i].mat->physicsType;
    long n = 0;
    if (rb) {
        C_Surface *s = rb->tex->sfc;
        *ox = (int)rb->x;
        *oy = (int)rb->y;
        *w = s->w;
        *h = s->h;
        n = (long)s->px.size();
        for (long i = 0; i < n && i < cap; i++) img[i] = s->px[(size_t)i];
        delete s;
        delete rb;
    }
    return n;
}
