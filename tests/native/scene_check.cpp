// scene_check.cpp -- host-side scene loading without a GPU: the scene-JSON/LMF
// loader (lt_json.cpp) and the host scene build (lt_scene.cpp) that
// lt_scene_load_json runs before anything reaches the device.
//
// Usage: scene_check <scene.json> ...
// For every file prints one line: "<status of load_scene_json> <status of
// build_host_scene or -1> <triangles> <lights> <light 0 radiance.x or 0>".
#include <stdio.h>

#include <string>

#include "lt_scene.h"

using namespace lt;

int main(int argc, char **argv) {
    for (int i = 1; i < argc; ++i) {
        lt_scene_desc desc;
        JsonSceneStorage storage;
        std::string err;
        const lt_status a = load_scene_json(argv[i], &desc, &storage, &err);
        int b = -1;
        size_t tris = 0, lights = 0;
        float rad = 0.0f;
        if (a == LT_OK) {
            HostScene hs;
            b = (int)build_host_scene(&desc, &hs, &err);
            if (b == LT_OK) {
                tris = hs.tri_geom.size();
                lights = hs.lights.size();
                if (lights) rad = hs.lights[0].radiance[0];
            }
        }
        printf("%d %d %zu %zu %.6g\n", (int)a, b, tris, lights, (double)rad);
    }
    return 0;
}
