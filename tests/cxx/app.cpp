// A reference-style application written against include/exposurerender.h:
// binds a texture, a plane light, a volume and a tracer, renders frames with
// RenderEstimate and reads the RGBA8 estimate with GetEstimate.
//
//   app <volume.raw> <res> <frames> <out.rgba>
//
// The scene constants are those of the 4-node blob workload of the Python
// scene builder (a 0.5 x 0.5 plane light at z = +1 facing down, multiplier 20,
// camera at (0,-2,0) looking at the origin, FOV 35, 40 x 32 film).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "exposurerender.h"

using namespace ExposureRender;

static int fail(const char* what) { std::fprintf(stderr, "FAIL: %s\n", what); return 1; }

int main(int argc, char** argv)
{
    if (argc < 5) return fail("usage");
    const int res = std::atoi(argv[2]);
    const int frames = std::atoi(argv[3]);
    std::vector<unsigned short> vox((size_t)res * res * res);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(vox.data(), 2, vox.size(), f) != vox.size()) return fail("volume read");
    std::fclose(f);

    ErTexture tex;
    tex.Procedural.UniformColor = ColorXYZf(1.0f, 1.0f, 1.0f);
    BindTexture(tex);
    if (tex.ID != 0) return fail("texture id");

    ErLight light;
    light.Visible = true;
    light.Shape.Type = Enums::Plane;
    light.Shape.Size = Vec3f(0.5f, 0.5f, 0.0f);
    const float m[4][4] = { { -1, 0, 0, 0 }, { 0, 1, 0, 0 }, { 0, 0, -1, 1 }, { 0, 0, 0, 1 } };
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) { light.Shape.TM.NN[i][j] = m[i][j]; light.Shape.InvTM.NN[i][j] = m[i][j]; }
    light.TextureID = tex.ID;
    light.Multiplier = 20.0f;
    BindLight(light);

    ErVolume volume;
    volume.BindVoxels(Vec3i(res, res, res), Vec3f(1.0f), vox.data(), true);
    BindVolume(volume);

    ErTracer tracer;
    tracer.Opacity1D.AddNode(ScalarNode(0.0f, 0.0f));
    tracer.Opacity1D.AddNode(ScalarNode(400.0f, 0.0f));
    tracer.Opacity1D.AddNode(ScalarNode(1500.0f, 0.6f));
    tracer.Opacity1D.AddNode(ScalarNode(4000.5f, 1.0f));
    const float dpos[4] = { 0.0f, 400.0f, 1500.0f, 4000.5f };
    const float dval[4][3] = { { 0.8f, 0.8f, 0.8f }, { 0.8f, 0.75f, 0.7f }, { 0.85f, 0.7f, 0.6f }, { 0.9f, 0.85f, 0.8f } };
    for (int k = 0; k < 4; k++) {
        ColorNode n;
        for (int c = 0; c < 3; c++) n.ScalarNodes[c] = ScalarNode(dpos[k], dval[k][c]);
        tracer.Diffuse1D.AddNode(n);
    }
    for (int k = 0; k < 2; k++) {
        ColorNode s, e;
        for (int c = 0; c < 3; c++) { s.ScalarNodes[c] = ScalarNode(k ? 4000.5f : 0.0f, 0.2f); e.ScalarNodes[c] = ScalarNode(k ? 4000.5f : 0.0f, 0.0f); }
        tracer.Specular1D.AddNode(s);
        tracer.Emission1D.AddNode(e);
        tracer.Glossiness1D.AddNode(ScalarNode(k ? 4000.5f : 0.0f, 0.6f));
    }
    tracer.Camera.FilmSize = Vec2i(40, 32);
    tracer.Camera.Pos = Vec3f(0.0f, -2.0f, 0.0f);
    tracer.Camera.Target = Vec3f(0.0f, 0.0f, 0.0f);
    tracer.Camera.Up = Vec3f(0.0f, 0.0f, 1.0f);
    tracer.VolumeID = volume.ID;
    tracer.LightIDs[0] = light.ID;
    tracer.LightIDs.Count = 1;
    BindTracer(tracer);

    bool threw = false;
    try { RenderEstimate(tracer.ID + 100); } catch (const Exception& e) { threw = e.Level == Enums::Warning; }
    if (!threw) return fail("unknown tracer did not throw");
    BindLight(light, false);
    BindLight(light, false);   // unknown ID: silent
    BindLight(light);          // rebinding gives a new ID (IDs are not reused)
    if (light.ID != 1) return fail("rebinding id");
    tracer.LightIDs[0] = light.ID;
    BindTracer(tracer);        // update in place

    for (int i = 0; i < frames; i++) RenderEstimate(tracer.ID);
    int n = -1;
    GetNoIterations(tracer.ID, n);
    if (n != frames) return fail("NoIterations");
    std::vector<unsigned char> rgba(40 * 32 * 4);
    GetEstimate(tracer.ID, rgba.data());
    FILE* o = std::fopen(argv[4], "wb");
    std::fwrite(rgba.data(), 1, rgba.size(), o);
    std::fclose(o);
    std::printf("ok tracer=%d volume=%d light=%d texture=%d\n", tracer.ID, volume.ID, light.ID, tex.ID);
    return 0;
}
