/*
 * er_cxx_api.cpp - the C++ entry points of include/exposurerender.h
 * (Source/exposurerender.h:32-42, Source/core.cu:50-155) over the C ABI.
 *
 * Error behaviour of the reference is kept: a full bind list and unbinding
 * an unknown item are silent (Source/list.cuh:63-67, :89-93), an unknown
 * tracer throws Exception(Warning, "...does not exist") (:150-164), CUDA and
 * other failures throw Exception(Error, message).
 */
#include <cstring>

#include "er_capi.h"
#include "exposurerender.h"

namespace ExposureRender
{

namespace
{

void raise(er_status st)
{
    if (st == ER_OK) return;
    const Enums::ExceptionLevel level = (st == ER_ERR_INVALID_ID) ? Enums::Warning : Enums::Error;
    throw Exception(level, er_last_error_message());
}

void to_plf(er_plf& o, const PiecewiseLinearFunction& p)
{
    std::memset(&o, 0, sizeof(o));
    o.count = p.Count;
    o.node_range[0] = p.NodeRange[0];
    o.node_range[1] = p.NodeRange[1];
    for (int i = 0; i < ER_MAX_TF_NODES; i++) {
        o.position[i] = p.Position[i];
        o.value[i] = p.Value[i];
    }
}

void to_ctf(er_color_tf& o, const ColorTransferFunction1D& t)
{
    for (int c = 0; c < 3; c++) to_plf(o.plf[c], t.PLF[c]);
}

void to_shape(er_shape& o, const Shape& s)
{
    std::memset(&o, 0, sizeof(o));
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            o.tm[i][j] = s.TM.NN[i][j];
            o.inv_tm[i][j] = s.InvTM.NN[i][j];
        }
    o.one_sided = s.OneSided ? 1 : 0;
    o.type = (int32_t)s.Type;
    for (int i = 0; i < 3; i++) o.size[i] = s.Size[i];
    o.area = s.Area;
    o.inner_radius = s.InnerRadius;
    o.outer_radius = s.OuterRadius;
}

/* Bind semantics of List::Bind (Source/list.cuh:59-83): a full list refuses silently */
template <class D, class F>
void bind(const ErBindable& item, const D& desc, F fn)
{
    int32_t id = item.ID;
    const er_status st = fn(&desc, &id);
    if (st == ER_ERR_LIST_FULL) return;
    raise(st);
    item.ID = id;
}

/* List::Unbind (Source/list.cuh:85-106): an unknown ID is ignored */
void unbind(er_status st)
{
    if (st == ER_ERR_INVALID_ID) return;
    raise(st);
}

}  // namespace

EXPOSURE_RENDER_DLL void BindTracer(const ErTracer& T, const bool& Bind)
{
    if (!Bind) { unbind(er_unbind_tracer(T.ID)); return; }
    er_tracer_desc d;
    std::memset(&d, 0, sizeof(d));
    to_plf(d.opacity, T.Opacity1D.PLF);
    to_ctf(d.diffuse, T.Diffuse1D);
    to_ctf(d.specular, T.Specular1D);
    to_plf(d.glossiness, T.Glossiness1D.PLF);
    to_ctf(d.emission, T.Emission1D);
    const Camera& c = T.Camera;
    d.camera.film_size[0] = c.FilmSize[0];
    d.camera.film_size[1] = c.FilmSize[1];
    for (int i = 0; i < 3; i++) {
        d.camera.pos[i] = c.Pos[i];
        d.camera.target[i] = c.Target[i];
        d.camera.up[i] = c.Up[i];
    }
    d.camera.focal_distance = c.FocalDistance;
    d.camera.aperture_size = c.ApertureSize;
    d.camera.clip_near = c.ClipNear;
    d.camera.clip_far = c.ClipFar;
    d.camera.exposure = c.Exposure;
    d.camera.gamma = c.Gamma;
    d.camera.fov = c.FOV;
    er_default_render_settings(&d.settings);
    const RenderSettings& r = T.RenderSettings;
    d.settings.step_factor_primary = r.Traversal.StepFactorPrimary;
    d.settings.step_factor_shadow = r.Traversal.StepFactorShadow;
    d.settings.shadows = r.Traversal.Shadows ? 1 : 0;
    d.settings.max_shadow_distance = r.Traversal.MaxShadowDistance;
    d.settings.shading_type = r.Shading.Type;
    d.settings.density_scale = r.Shading.DensityScale;
    d.settings.opacity_modulated = r.Shading.OpacityModulated ? 1 : 0;
    d.settings.gradient_computation = r.Shading.GradientComputation;
    d.settings.gradient_threshold = r.Shading.GradientThreshold;
    d.settings.gradient_factor = r.Shading.GradientFactor;
    d.settings.apply_shading_type = r.Extensions.ApplyShadingType ? 1 : 0;
    d.settings.free_flight = r.Extensions.FreeFlight;
    d.settings.mis = r.Extensions.Mis;
    d.settings.volume_ior = r.Extensions.VolumeIor;
    d.settings.frame_filter = r.Extensions.FrameFilter ? 1 : -1;
    d.settings.bilateral = r.Extensions.Bilateral ? 1 : 0;
    d.settings.bilateral_radius = r.Extensions.BilateralRadius;
    d.settings.bilateral_sigma_d = r.Extensions.BilateralSigmaD;
    d.settings.bilateral_sigma_r = r.Extensions.BilateralSigmaR;
    d.settings.seed = r.Extensions.Seed;
    d.settings.majorant_brick = r.Extensions.MajorantBrick;
    d.settings.stratify = r.Extensions.Stratify ? 1 : 0;
    d.volume_id = T.VolumeID;
    d.light_count = T.LightIDs.Count;
    d.object_count = T.ObjectIDs.Count;
    d.clipping_object_count = T.ClippingObjectIDs.Count;
    for (int i = 0; i < ER_MAX_INDICES; i++) {
        d.light_ids[i] = T.LightIDs.D[i];
        d.object_ids[i] = T.ObjectIDs.D[i];
        d.clipping_object_ids[i] = T.ClippingObjectIDs.D[i];
    }
    bind(T, d, er_bind_tracer);
}

EXPOSURE_RENDER_DLL void BindVolume(const ErVolume& V, const bool& Bind)
{
    if (!Bind) { unbind(er_unbind_volume(V.ID)); return; }
    er_volume_desc d;
    std::memset(&d, 0, sizeof(d));
    for (int i = 0; i < 3; i++) {
        d.resolution[i] = V.Resolution[i];
        d.spacing[i] = V.Spacing[i];
    }
    d.normalize_size = V.NormalizeSize ? 1 : 0;
    d.voxels = V.Voxels.empty() ? nullptr : V.Voxels.data();
    bind(V, d, er_bind_volume);
}

EXPOSURE_RENDER_DLL void BindLight(const ErLight& L, const bool& Bind)
{
    if (!Bind) { unbind(er_unbind_light(L.ID)); return; }
    er_light_desc d;
    std::memset(&d, 0, sizeof(d));
    d.visible = L.Visible ? 1 : 0;
    to_shape(d.shape, L.Shape);
    d.texture_id = L.TextureID;
    d.multiplier = L.Multiplier;
    d.unit = (int32_t)L.Unit;
    bind(L, d, er_bind_light);
}

EXPOSURE_RENDER_DLL void BindObject(const ErObject& O, const bool& Bind)
{
    if (!Bind) { unbind(er_unbind_object(O.ID)); return; }
    er_object_desc d;
    std::memset(&d, 0, sizeof(d));
    to_shape(d.shape, O.Shape);
    d.diffuse_texture_id = O.DiffuseTextureID;
    d.specular_texture_id = O.SpecularTextureID;
    d.glossiness_texture_id = O.GlossinessTextureID;
    d.ior = O.Ior;
    bind(O, d, er_bind_object);
}

EXPOSURE_RENDER_DLL void BindClippingObject(const ErClippingObject& C, const bool& Bind)
{
    if (!Bind) { unbind(er_unbind_clipping_object(C.ID)); return; }
    er_clipping_object_desc d;
    std::memset(&d, 0, sizeof(d));
    to_shape(d.shape, C.Shape);
    d.invert = C.Invert ? 1 : 0;
    bind(C, d, er_bind_clipping_object);
}

EXPOSURE_RENDER_DLL void BindTexture(const ErTexture& T, const bool& Bind)
{
    if (!Bind) { unbind(er_unbind_texture(T.ID)); return; }
    er_texture_desc d;
    std::memset(&d, 0, sizeof(d));
    d.type = (int32_t)T.Type;
    d.output_level = T.OutputLevel;
    d.bitmap_id = T.BitmapID;
    d.procedural.type = (int32_t)T.Procedural.Type;
    for (int i = 0; i < 3; i++) {
        d.procedural.uniform_color[i] = T.Procedural.UniformColor[i];
        d.procedural.checker_color1[i] = T.Procedural.CheckerColor1[i];
        d.procedural.checker_color2[i] = T.Procedural.CheckerColor2[i];
    }
    to_ctf(d.procedural.gradient, T.Procedural.Gradient);
    d.offset[0] = T.Offset[0];
    d.offset[1] = T.Offset[1];
    d.repeat[0] = T.Repeat[0];
    d.repeat[1] = T.Repeat[1];
    d.flip[0] = T.Flip[0];
    d.flip[1] = T.Flip[1];
    bind(T, d, er_bind_texture);
}

EXPOSURE_RENDER_DLL void BindBitmap(const ErBitmap& B, const bool& Bind)
{
    if (!Bind) { unbind(er_unbind_bitmap(B.ID)); return; }
    er_bitmap_desc d;
    std::memset(&d, 0, sizeof(d));
    d.resolution[0] = B.Resolution[0];
    d.resolution[1] = B.Resolution[1];
    d.pixels = B.Pixels.empty() ? nullptr : reinterpret_cast<const uint8_t*>(B.Pixels.data());
    bind(B, d, er_bind_bitmap);
}

EXPOSURE_RENDER_DLL void RenderEstimate(int TracerID) { raise(er_render_estimate(TracerID)); }

EXPOSURE_RENDER_DLL void GetEstimate(int TracerID, unsigned char* pData) { raise(er_get_estimate(TracerID, pData)); }

EXPOSURE_RENDER_DLL void GetAutoFocusDistance(int TracerID, int FilmU, int FilmV, float& AutoFocusDistance)
{
    raise(er_get_auto_focus_distance(TracerID, FilmU, FilmV, &AutoFocusDistance));
}

EXPOSURE_RENDER_DLL void GetNoIterations(int TracerID, int& NoIterations)
{
    int32_t n = 0;
    raise(er_get_no_iterations(TracerID, &n));
    NoIterations = n;
}

}  // namespace ExposureRender
