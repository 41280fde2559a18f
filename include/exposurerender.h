/*
 * exposurerender.h - C++ API of the GB300 transport library, source-compatible
 * with the reference's Source/exposurerender.h:32-42.
 *
 * The eleven entry points keep their names and signatures (namespace
 * ExposureRender, exported from libexposurerender.so with default
 * visibility).  The Er* types keep the public fields, defaults and helpers a
 * reference application uses (AddNode, BindVoxels, BindPixels, Camera
 * fields, RenderSettings, LightIDs, the mutable ID written by Bind); their
 * binary layout is not the reference's (which carries vtables and device
 * buffers), so applications are recompiled against this header.
 *
 * Behaviour follows Source/core.cu and Source/list.cuh: binding assigns
 * ID = counter++ through the mutable ID, rebinding an existing ID updates it,
 * a full list (31 items) refuses silently, unbinding an unknown ID is
 * silent, and rendering or reading an unknown tracer throws
 * ExposureRender::Exception(Warning, "... does not exist").  CUDA failures
 * throw Exception(Error, ...).  Each call maps onto one er_* function of
 * er_capi.h.
 */
#ifndef EXPOSURERENDER_H
#define EXPOSURERENDER_H

#include <cfloat>
#include <cstring>
#include <vector>

#if defined(_WIN32)
#define EXPOSURE_RENDER_DLL __declspec(dllexport)
#else
#define EXPOSURE_RENDER_DLL __attribute__((visibility("default")))
#endif

namespace ExposureRender
{

/* Source/enums.h:24-108 */
namespace Enums
{
    enum MemoryType { Host, Device };
    enum ProceduralType { Uniform = 0, Checker, Gradient };
    enum TextureType { Procedural = 0, Bitmap };
    enum ShapeType { Plane = 0, Disk, Ring, Box, Sphere, Cylinder, Cone };
    enum ShadingMode { BrdfOnly = 0, PhaseFunctionOnly, Hybrid, Modulation, Threshold, GradientMagnitude };
    enum GradientMode { ForwardDifferences = 0, CentralDifferences, Filtered };
    enum ExceptionLevel { Info = 0, Warning, Error, Fatal };
    enum EmissionUnit { Power = 0, Lux, Intensity };
    enum ScatterFunction { Brdf, PhaseFunction };
    enum ScatterType { Volume, Light, Object, SlicePlane };
}

/* Source/exception.h:27-55 */
class EXPOSURE_RENDER_DLL Exception
{
public:
    Exception(const Enums::ExceptionLevel& Level, const char* pMessage = "") : Level(Level)
    {
        std::strncpy(this->Message, pMessage ? pMessage : "", sizeof(this->Message) - 1);
        this->Message[sizeof(this->Message) - 1] = 0;
    }
    Enums::ExceptionLevel Level;
    char Message[256];
};

/* small vectors (Source/vector.h:397-519) */
template <class T, int N>
class Vec
{
public:
    Vec() { for (int i = 0; i < N; i++) D[i] = T(0); }
    explicit Vec(const T& v) { for (int i = 0; i < N; i++) D[i] = v; }
    T operator[](const int& i) const { return D[i]; }
    T& operator[](const int& i) { return D[i]; }
    T D[N];
};

class Vec2i : public Vec<int, 2> { public: Vec2i() {} explicit Vec2i(int v) : Vec<int, 2>(v) {} Vec2i(int a, int b) { D[0] = a; D[1] = b; } };
class Vec2f : public Vec<float, 2> { public: Vec2f() {} explicit Vec2f(float v) : Vec<float, 2>(v) {} Vec2f(float a, float b) { D[0] = a; D[1] = b; } };
class Vec3i : public Vec<int, 3> { public: Vec3i() {} explicit Vec3i(int v) : Vec<int, 3>(v) {} Vec3i(int a, int b, int c) { D[0] = a; D[1] = b; D[2] = c; } };
class Vec3f : public Vec<float, 3> { public: Vec3f() {} explicit Vec3f(float v) : Vec<float, 3>(v) {} Vec3f(float a, float b, float c) { D[0] = a; D[1] = b; D[2] = c; } };
class ColorXYZf : public Vec<float, 3> { public: ColorXYZf() {} explicit ColorXYZf(float v) : Vec<float, 3>(v) {} ColorXYZf(float a, float b, float c) { D[0] = a; D[1] = b; D[2] = c; } };

class ColorRGBAuc : public Vec<unsigned char, 4>
{
public:
    ColorRGBAuc() {}
    ColorRGBAuc(unsigned char r, unsigned char g, unsigned char b, unsigned char a) { D[0] = r; D[1] = g; D[2] = b; D[3] = a; }
};

/* Source/matrix.h:27-56 */
class EXPOSURE_RENDER_DLL Matrix44
{
public:
    Matrix44() { for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) NN[i][j] = i == j ? 1.0f : 0.0f; }
    float NN[4][4];
};

/* Source/vector.h:554-579 */
class EXPOSURE_RENDER_DLL Indices
{
public:
    Indices() : Count(0) { for (int i = 0; i < 256; i++) D[i] = -1; }
    int operator[](const int& i) const { return D[i]; }
    int& operator[](const int& i) { return D[i]; }
    int D[256];
    int Count;
};

/* Source/plf.h:26-92, Source/pf.h:35-71 */
class EXPOSURE_RENDER_DLL PiecewiseLinearFunction
{
public:
    PiecewiseLinearFunction() : NodeRange(FLT_MAX, FLT_MIN), Count(0)
    {
        for (int i = 0; i < 128; i++) { Position[i] = 0.0f; Value[i] = 0.0f; }
    }
    void AddNode(const float& P, const float& V)
    {
        if (Count + 1 >= 128) return;
        Position[Count] = P;
        Value[Count] = V;
        if (P < NodeRange[0]) NodeRange[0] = P;
        if (P > NodeRange[1]) NodeRange[1] = P;
        Count++;
    }
    Vec2f NodeRange;
    float Position[128];
    float Value[128];
    int Count;
};

/* Source/transferfunction.h:27-154 */
class EXPOSURE_RENDER_DLL ScalarNode
{
public:
    ScalarNode() : Position(0.0f), Value(0.0f) {}
    ScalarNode(float Position, float Value) : Position(Position), Value(Value) {}
    float Position;
    float Value;
};

class EXPOSURE_RENDER_DLL ColorNode
{
public:
    ScalarNode ScalarNodes[3];
};

class EXPOSURE_RENDER_DLL ScalarTransferFunction1D
{
public:
    void AddNode(const ScalarNode& Node) { PLF.AddNode(Node.Position, Node.Value); }
    PiecewiseLinearFunction PLF;
};

class EXPOSURE_RENDER_DLL ColorTransferFunction1D
{
public:
    void AddNode(const ColorNode& Node)
    {
        for (int i = 0; i < 3; i++) PLF[i].AddNode(Node.ScalarNodes[i].Position, Node.ScalarNodes[i].Value);
    }
    PiecewiseLinearFunction PLF[3];
};

/* Source/erbindable.h:28-68 */
class EXPOSURE_RENDER_DLL ErBindable
{
public:
    ErBindable() : ID(-1), Enabled(true), Dirty(false) {}
    virtual ~ErBindable() {}
    mutable int ID;
    bool Enabled;
    bool Dirty;
};

/* Source/shape.h:57-113 */
class EXPOSURE_RENDER_DLL Shape
{
public:
    Shape() : OneSided(false), Type(Enums::Plane), Area(0.0f), InnerRadius(0.0f), OuterRadius(0.0f) {}
    Matrix44 TM;
    Matrix44 InvTM;
    bool OneSided;
    Enums::ShapeType Type;
    Vec3f Size;
    float Area;
    float InnerRadius;
    float OuterRadius;
};

/* Source/ervolume.h:28-74 */
class EXPOSURE_RENDER_DLL ErVolume : public ErBindable
{
public:
    ErVolume() : NormalizeSize(false), Spacing(1.0f) {}
    void BindVoxels(const Vec3i& Resolution, const Vec3f& Spacing, unsigned short* Voxels, const bool& NormalizeSize = false)
    {
        this->Resolution = Resolution;
        const size_t n = (size_t)Resolution[0] * (size_t)Resolution[1] * (size_t)Resolution[2];
        this->Voxels.assign(Voxels, Voxels + n);
        this->NormalizeSize = NormalizeSize;
        this->Spacing = Spacing;
    }
    Vec3i Resolution;
    std::vector<unsigned short> Voxels;
    bool NormalizeSize;
    Vec3f Spacing;
};

/* Source/erlight.h:27-66 */
class EXPOSURE_RENDER_DLL ErLight : public ErBindable
{
public:
    ErLight() : Visible(false), TextureID(-1), Multiplier(0.0f), Unit(Enums::Power) {}
    bool Visible;
    ExposureRender::Shape Shape;
    int TextureID;
    float Multiplier;
    Enums::EmissionUnit Unit;
};

/* Source/procedural.h:27-60 */
class EXPOSURE_RENDER_DLL Procedural
{
public:
    Procedural() : Type(Enums::Uniform) {}
    Enums::ProceduralType Type;
    ColorXYZf UniformColor;
    ColorXYZf CheckerColor1;
    ColorXYZf CheckerColor2;
    ColorTransferFunction1D Gradient;
};

/* Source/ertexture.h:27-82 */
class EXPOSURE_RENDER_DLL ErTexture : public ErBindable
{
public:
    ErTexture() : Type(Enums::Procedural), OutputLevel(1.0f), BitmapID(-1), Offset(0.0f), Repeat(0.0f), Flip(0) {}
    Enums::TextureType Type;
    float OutputLevel;
    int BitmapID;
    ExposureRender::Procedural Procedural;
    Vec2f Offset;
    Vec2f Repeat;
    Vec2i Flip;
};

/* Source/erbitmap.h:28-61 */
class EXPOSURE_RENDER_DLL ErBitmap : public ErBindable
{
public:
    void BindPixels(const Vec2i& Resolution, ColorRGBAuc* Pixels)
    {
        this->Resolution = Resolution;
        const size_t n = (size_t)Resolution[0] * (size_t)Resolution[1];
        this->Pixels.assign(Pixels, Pixels + n);
    }
    Vec2i Resolution;
    std::vector<ColorRGBAuc> Pixels;
};

/* Source/erobject.h:27-67 */
class EXPOSURE_RENDER_DLL ErObject : public ErBindable
{
public:
    ErObject() : DiffuseTextureID(-1), SpecularTextureID(-1), GlossinessTextureID(-1), Ior(5.0f) {}
    ExposureRender::Shape Shape;
    int DiffuseTextureID;
    int SpecularTextureID;
    int GlossinessTextureID;
    float Ior;
};

/* Source/erclippingobject.h:27-58 */
class EXPOSURE_RENDER_DLL ErClippingObject : public ErBindable
{
public:
    ErClippingObject() : Invert(false) {}
    ExposureRender::Shape Shape;
    bool Invert;
};

/* Source/camera.h:26-116 (inputs; the derived frame is computed by the library) */
class EXPOSURE_RENDER_DLL Camera
{
public:
    Camera() : FocalDistance(-1.0f), ApertureSize(0.0f), ClipNear(0.0f), ClipFar(1000.0f), Exposure(1.0f), Gamma(2.2f), FOV(35.0f) {}
    Vec2i FilmSize;
    Vec3f Pos;
    Vec3f Target;
    Vec3f Up;
    float FocalDistance;
    float ApertureSize;
    float ClipNear;
    float ClipFar;
    float Exposure;
    float Gamma;
    float FOV;
};

/* Source/rendersettings.h:27-131, plus the extension switches of er_capi.h */
class EXPOSURE_RENDER_DLL RenderSettings
{
public:
    class EXPOSURE_RENDER_DLL TraversalSettings
    {
    public:
        TraversalSettings() : StepFactorPrimary(0.1f), StepFactorShadow(0.1f), Shadows(true), MaxShadowDistance(1.0f) {}
        float StepFactorPrimary;
        float StepFactorShadow;
        bool Shadows;
        float MaxShadowDistance;
    };

    class EXPOSURE_RENDER_DLL ShadingSettings
    {
    public:
        ShadingSettings() : Type(0), DensityScale(100.0f), OpacityModulated(true), GradientComputation(1), GradientThreshold(0.5f),
                            GradientFactor(0.5f) {}
        int Type;
        float DensityScale;
        bool OpacityModulated;
        int GradientComputation;
        float GradientThreshold;
        float GradientFactor;
    };

    class EXPOSURE_RENDER_DLL ExtensionSettings
    {
    public:
        ExtensionSettings() : ApplyShadingType(false), FreeFlight(0), Mis(0), VolumeIor(15.0f), FrameFilter(true), Bilateral(false),
                              BilateralRadius(2), BilateralSigmaD(1.5f), BilateralSigmaR(20.0f), Seed(1u), MajorantBrick(8),
                              Stratify(false) {}
        bool ApplyShadingType;   /* Shading.Type selects BRDF / phase / hybrid (Source/scatterevent.h:155-212) */
        int FreeFlight;          /* 0 fixed-step march (reference), 1 delta tracking */
        int Mis;                 /* 0 light sampling (reference), 1 light + BSDF sampling */
        float VolumeIor;
        bool FrameFilter;
        bool Bilateral;
        int BilateralRadius;
        float BilateralSigmaD;
        float BilateralSigmaR;
        unsigned int Seed;
        int MajorantBrick;
        bool Stratify;           /* multi-sample renders: light, BSDF and first free-flight samples from per-pixel shifted lattices */
    };

    TraversalSettings Traversal;
    ShadingSettings Shading;
    ExtensionSettings Extensions;
};

/* Source/ertracer.h:33-117 */
class EXPOSURE_RENDER_DLL ErTracer : public ErBindable
{
public:
    ErTracer() : NoIterations(0), VolumeID(0) {}
    ScalarTransferFunction1D Opacity1D;
    ColorTransferFunction1D Diffuse1D;
    ColorTransferFunction1D Specular1D;
    ScalarTransferFunction1D Glossiness1D;
    ColorTransferFunction1D Emission1D;
    ExposureRender::Camera Camera;
    ExposureRender::RenderSettings RenderSettings;
    int NoIterations;
    int VolumeID;
    Indices LightIDs;
    Indices ObjectIDs;
    Indices ClippingObjectIDs;
};

/* Source/exposurerender.h:32-42 */
EXPOSURE_RENDER_DLL void BindTracer(const ErTracer& Tracer, const bool& Bind = true);
EXPOSURE_RENDER_DLL void BindVolume(const ErVolume& Volume, const bool& Bind = true);
EXPOSURE_RENDER_DLL void BindLight(const ErLight& Light, const bool& Bind = true);
EXPOSURE_RENDER_DLL void BindObject(const ErObject& Object, const bool& Bind = true);
EXPOSURE_RENDER_DLL void BindClippingObject(const ErClippingObject& ClippingObject, const bool& Bind = true);
EXPOSURE_RENDER_DLL void BindTexture(const ErTexture& Texture, const bool& Bind = true);
EXPOSURE_RENDER_DLL void BindBitmap(const ErBitmap& Bitmap, const bool& Bind = true);
EXPOSURE_RENDER_DLL void RenderEstimate(int TracerID);
EXPOSURE_RENDER_DLL void GetEstimate(int TracerID, unsigned char* pData);
EXPOSURE_RENDER_DLL void GetAutoFocusDistance(int TracerID, int FilmU, int FilmV, float& AutoFocusDistance);
EXPOSURE_RENDER_DLL void GetNoIterations(int TracerID, int& NoIterations);

}  // namespace ExposureRender

#endif
