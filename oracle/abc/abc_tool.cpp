// abc_tool — test infrastructure for the Alembic scene front-end.
//
// Built against the reference's vendored Alembic library and its
// houdini_alembic reader (libs/abc, libs/houdini_alembic), compiled from
// their sources by oracle/build_oracle.py into oracle/_ref/abc_tool.
//
//   abc_tool write <out.abc> <scene>   writes one of the synthetic test scenes
//                                      below with the Alembic writer API, shaped
//                                      like a Houdini export (transform parents,
//                                      "material" and property columns as
//                                      geometry parameters, a camera with
//                                      resx/resy user properties, point objects)
//   abc_tool dump <in.abc> <frame>     reads the file with
//                                      houdini_alembic::AlembicStorage (what
//                                      WavefrontPathTracing uses,
//                                      common/wavefront_path_tracing.hpp:1170-1216)
//                                      and prints every object it returns as JSON
//
// The dump is the oracle the library's own Alembic reader is checked against.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <Alembic/Abc/All.h>
#include <Alembic/AbcCoreOgawa/All.h>
#include <Alembic/AbcGeom/All.h>

#include "houdini_alembic.hpp"

using namespace Alembic::Abc;
using namespace Alembic::AbcGeom;

namespace {

// ---------------------------------------------------------------- writing
uint32_t g_state = 12345u;
float rnd() {  // LCG in [0, 1)
    g_state = g_state * 1664525u + 1013904223u;
    return (float)(g_state >> 8) * (1.0f / 16777216.0f);
}

void set_visibility(OObject& o, int8_t v) {
    OVisibilityProperty vis = CreateVisibilityProperty(o, 0);
    vis.set(v);
}

struct MeshSpec {
    std::vector<V3f> P;
    std::vector<int32_t> idx, cnt;
};

MeshSpec grid_mesh(int nx, int ny, float z, bool quads) {
    MeshSpec m;
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i)
            m.P.push_back(V3f(-1.0f + 2.0f * i / nx, -1.0f + 2.0f * j / ny, z + 0.05f * std::sin(3.0f * i + 2.0f * j)));
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int a = j * (nx + 1) + i, b = a + 1, c = a + nx + 1, d = c + 1;
            if (quads) {
                m.idx.insert(m.idx.end(), {a, b, d, c});
                m.cnt.push_back(4);
            } else {
                m.idx.insert(m.idx.end(), {a, b, d, a, d, c});
                m.cnt.insert(m.cnt.end(), {3, 3});
            }
        }
    return m;
}

// per-face material columns in the shape Houdini writes them
void write_material_columns(OCompoundProperty arb, size_t nf, const char* const* names, int nnames,
                            bool cd_as_array_extent) {
    std::vector<std::string> vals(names, names + nnames);
    std::vector<uint32_t> which(nf);
    for (size_t f = 0; f < nf; ++f) which[f] = (uint32_t)(f % nnames);
    OStringGeomParam mat(arb, "material", true, kUniformScope, 1);
    mat.set(OStringGeomParam::Sample(StringArraySample(vals), UInt32ArraySample(which), kUniformScope));

    std::vector<C3f> cd(nf), le(nf);
    std::vector<V3f> refl(nf), tint(nf);
    std::vector<float> alpha(nf), falloff(nf), C(nf), cdflat(3 * nf);
    std::vector<int32_t> back(nf);
    for (size_t f = 0; f < nf; ++f) {
        cd[f] = C3f(rnd(), rnd(), rnd());
        le[f] = (f % 7 == 0) ? C3f(4.0f * rnd(), 3.0f * rnd(), 2.0f * rnd()) : C3f(0, 0, 0);
        refl[f] = V3f(rnd(), rnd(), rnd());
        tint[f] = V3f(rnd(), rnd(), rnd());
        alpha[f] = 0.05f + 0.45f * rnd();
        falloff[f] = rnd();
        C[f] = 0.2f + rnd();
        back[f] = (int32_t)(f % 3 == 0);
        cdflat[3 * f] = cd[f].x;
        cdflat[3 * f + 1] = cd[f].y;
        cdflat[3 * f + 2] = cd[f].z;
    }
    if (cd_as_array_extent) {  // a float tuple of arrayExtent 3, as Houdini writes vector attributes
        OFloatGeomParam p(arb, "Cd", false, kUniformScope, 3);
        p.set(OFloatGeomParam::Sample(FloatArraySample(cdflat), kUniformScope));
    } else {
        OC3fGeomParam p(arb, "Cd", false, kUniformScope, 1);
        p.set(OC3fGeomParam::Sample(C3fArraySample(cd), kUniformScope));
    }
    OC3fGeomParam pLe(arb, "Le", false, kUniformScope, 1);
    pLe.set(OC3fGeomParam::Sample(C3fArraySample(le), kUniformScope));
    OV3fGeomParam pr(arb, "reflectance", false, kUniformScope, 1);
    pr.set(OV3fGeomParam::Sample(V3fArraySample(refl), kUniformScope));
    OV3fGeomParam pt(arb, "edgetint", false, kUniformScope, 1);
    pt.set(OV3fGeomParam::Sample(V3fArraySample(tint), kUniformScope));
    OFloatGeomParam pa(arb, "alpha", false, kUniformScope, 1);
    pa.set(OFloatGeomParam::Sample(FloatArraySample(alpha), kUniformScope));
    OFloatGeomParam pf(arb, "falloff", false, kUniformScope, 1);
    pf.set(OFloatGeomParam::Sample(FloatArraySample(falloff), kUniformScope));
    OFloatGeomParam pc(arb, "C", false, kUniformScope, 1);
    pc.set(OFloatGeomParam::Sample(FloatArraySample(C), kUniformScope));
    OInt32GeomParam pb(arb, "BackEmission", false, kUniformScope, 1);
    pb.set(OInt32GeomParam::Sample(Int32ArraySample(back), kUniformScope));
}

OPolyMesh write_mesh(OObject parent, const char* name, const MeshSpec& m) {
    OPolyMesh mesh(parent, name);
    OPolyMeshSchema::Sample s(P3fArraySample(m.P), Int32ArraySample(m.idx), Int32ArraySample(m.cnt));
    mesh.getSchema().set(s);
    return mesh;
}

void write_basic(const char* path) {
    OArchive archive(Alembic::AbcCoreOgawa::WriteArchive(), path);
    OObject top = archive.getTop();
    static const char* const kNames[] = {"Lambertian", "Ward", "Dierectric", "HomogeneousVolume", "Specular"};

    // translate, rotate about y, non-uniform scale; a triangle grid with every column
    OXform xf(top, "mesh_xf");
    XformSample xs;
    xs.setTranslation(V3d(1.0, 2.0, 3.0));
    xs.setYRotation(30.0);
    xs.setScale(V3d(2.0, 1.5, 0.5));
    xf.getSchema().set(xs);
    set_visibility(xf, -1);
    MeshSpec m = grid_mesh(3, 2, 0.0f, false);
    OPolyMesh mesh = write_mesh(xf, "mesh", m);
    OCompoundProperty arb = mesh.getSchema().getArbGeomParams();
    write_material_columns(arb, m.cnt.size(), kNames, 5, false);
    {  // a per-point float, a face-varying indexed uv, a plain V2f (the reader drops it), a string
        std::vector<float> w(m.P.size());
        for (size_t i = 0; i < w.size(); ++i) w[i] = 0.5f * (float)i;
        OFloatGeomParam pw(arb, "pweight", false, kVaryingScope, 1);
        pw.set(OFloatGeomParam::Sample(FloatArraySample(w), kVaryingScope));
        std::vector<V2f> uvv = {V2f(0, 0), V2f(1, 0), V2f(1, 1), V2f(0, 1)};
        std::vector<uint32_t> uvi(m.idx.size());
        for (size_t i = 0; i < uvi.size(); ++i) uvi[i] = (uint32_t)(i % 4);
        OV2fGeomParam uv(arb, "uv", true, kFacevaryingScope, 1);
        uv.set(OV2fGeomParam::Sample(V2fArraySample(uvv), UInt32ArraySample(uvi), kFacevaryingScope));
        std::vector<V2f> st(m.cnt.size(), V2f(0.25f, 0.75f));
        OV2fGeomParam pst(arb, "st", false, kUniformScope, 1);
        pst.set(OV2fGeomParam::Sample(V2fArraySample(st), kUniformScope));
        std::vector<std::string> tags(m.cnt.size());
        for (size_t f = 0; f < tags.size(); ++f) tags[f] = "face" + std::to_string(f);
        OStringGeomParam ptag(arb, "tag", false, kUniformScope, 1);
        ptag.set(OStringGeomParam::Sample(StringArraySample(tags), kUniformScope));
    }
    // nested transform: a child grid whose parent is mesh_xf
    OXform child(xf, "child_xf");
    XformSample cs;
    cs.setRotation(V3d(1.0, 1.0, 0.0), 45.0);
    cs.setTranslation(V3d(0.0, 0.5, 0.0));
    child.getSchema().set(cs);
    MeshSpec m2 = grid_mesh(2, 2, 0.3f, false);
    OPolyMesh mesh2 = write_mesh(child, "child_mesh", m2);
    static const char* const kLamb[] = {"Lambertian"};
    write_material_columns(mesh2.getSchema().getArbGeomParams(), m2.cnt.size(), kLamb, 1, true);

    // a matrix op and a quad mesh (not a triangle mesh: the scene skips it)
    OXform qxf(top, "quad_xf");
    XformSample qs;
    M44d mat;
    mat.makeIdentity();
    mat[0][0] = 0.9;
    mat[0][1] = 0.1;
    mat[1][0] = -0.1;
    mat[1][1] = 0.9;
    mat[3][0] = -2.0;
    mat[3][2] = 0.25;
    qs.setMatrix(mat);
    qxf.getSchema().set(qs);
    // (every mesh gets geometry parameters: the Houdini reader dereferences them unconditionally)
    static const char* const kLamb1[] = {"Lambertian"};
    MeshSpec mq = grid_mesh(2, 1, -0.5f, true);
    write_material_columns(write_mesh(qxf, "quads", mq).getSchema().getArbGeomParams(), mq.cnt.size(), kLamb1, 1,
                           false);

    // hidden (0) and "visible" (1) parents: the Houdini reader counts only -1 (deferred) as visible
    OXform hxf(top, "hidden_xf");
    XformSample ident;
    hxf.getSchema().set(ident);
    set_visibility(hxf, 0);
    MeshSpec mh = grid_mesh(1, 1, 2.0f, false);
    write_material_columns(write_mesh(hxf, "hidden_mesh", mh).getSchema().getArbGeomParams(), mh.cnt.size(), kLamb1,
                           1, false);
    OXform vxf(top, "vis1_xf");
    vxf.getSchema().set(ident);
    set_visibility(vxf, 1);
    MeshSpec mv = grid_mesh(1, 1, 3.0f, false);
    write_material_columns(write_mesh(vxf, "vis1_mesh", mv).getSchema().getArbGeomParams(), mv.cnt.size(), kLamb1,
                           1, false);

    // spheres: a point object with pscale and Cd
    OXform pxf(top, "spheres_xf");
    XformSample ps;
    ps.setTranslation(V3d(0.0, 0.0, -1.0));
    pxf.getSchema().set(ps);
    OPoints pts(pxf, "spheres");
    std::vector<V3f> pp = {V3f(0.1f, 0.2f, 0.3f), V3f(-0.5f, 0.25f, 0.0f), V3f(0.7f, -0.4f, 0.2f)};
    std::vector<uint64_t> ids = {0, 1, 2};
    pts.getSchema().set(OPointsSchema::Sample(P3fArraySample(pp), UInt64ArraySample(ids)));
    {
        OCompoundProperty parb = pts.getSchema().getArbGeomParams();
        std::vector<float> ps3 = {0.1f, 0.2f, 0.15f};
        OFloatGeomParam pscale(parb, "pscale", false, kVaryingScope, 1);
        pscale.set(OFloatGeomParam::Sample(FloatArraySample(ps3), kVaryingScope));
        std::vector<C3f> cd = {C3f(0.9f, 0.1f, 0.1f), C3f(0.1f, 0.9f, 0.1f), C3f(0.1f, 0.1f, 0.9f)};
        OC3fGeomParam pcd(parb, "Cd", false, kVaryingScope, 1);
        pcd.set(OC3fGeomParam::Sample(C3fArraySample(cd), kVaryingScope));
    }

    // the environment: a one-point object whose point_type is ImageEnvmap
    OXform exf(top, "env_xf");
    exf.getSchema().set(ident);
    OPoints env(exf, "env");
    std::vector<V3f> ep = {V3f(0, 0, 0)};
    std::vector<uint64_t> eid = {0};
    env.getSchema().set(OPointsSchema::Sample(P3fArraySample(ep), UInt64ArraySample(eid)));
    {
        OCompoundProperty earb = env.getSchema().getArbGeomParams();
        std::vector<std::string> pt = {"ImageEnvmap"}, file = {"sky_tiny.hdr"};
        OStringGeomParam ptype(earb, "point_type", false, kVaryingScope, 1);
        ptype.set(OStringGeomParam::Sample(StringArraySample(pt), kVaryingScope));
        OStringGeomParam pfile(earb, "file", false, kVaryingScope, 1);
        pfile.set(OStringGeomParam::Sample(StringArraySample(file), kVaryingScope));
        std::vector<float> clamp = {50.0f}, scale = {2.0f};
        OFloatGeomParam pclamp(earb, "clamp", false, kVaryingScope, 1);
        pclamp.set(OFloatGeomParam::Sample(FloatArraySample(clamp), kVaryingScope));
        OFloatGeomParam pscale(earb, "scale", false, kVaryingScope, 1);
        pscale.set(OFloatGeomParam::Sample(FloatArraySample(scale), kVaryingScope));
    }

    // the camera, under a transform, with Houdini's resx / resy user properties
    OXform cxf(top, "cam_xf");
    XformSample cxs;
    cxs.setTranslation(V3d(0.0, 1.0, 6.0));
    cxs.setXRotation(-8.0);
    cxf.getSchema().set(cxs);
    OCamera cam(cxf, "cam");
    CameraSample csmp;
    csmp.setFocalLength(35.0);
    csmp.setHorizontalAperture(3.6);
    csmp.setVerticalAperture(2.4);
    csmp.setFocusDistance(6.0);
    csmp.setFStop(8.0);
    csmp.setNearClippingPlane(0.01);
    csmp.setFarClippingPlane(1000.0);
    cam.getSchema().set(csmp);
    OCompoundProperty up = cam.getSchema().getUserProperties();
    OFloatProperty resx(up, "resx"), resy(up, "resy");
    resx.set(64.0f);
    resy.set(48.0f);
}

// A larger scene for rendering: a displaced grid of random materials (no
// volumes, no delta materials behind glass), a light panel, spheres, camera.
void write_render(const char* path) {
    g_state = 777u;
    OArchive archive(Alembic::AbcCoreOgawa::WriteArchive(), path);
    OObject top = archive.getTop();
    static const char* const kNames[] = {"Lambertian", "Ward", "Lambertian", "Specular", "Dierectric"};
    OXform xf(top, "floor_xf");
    XformSample xs;
    xs.setXRotation(-90.0);
    xs.setScale(V3d(3.0, 3.0, 1.0));
    xf.getSchema().set(xs);
    MeshSpec m = grid_mesh(16, 16, 0.0f, false);
    OPolyMesh mesh = write_mesh(xf, "floor", m);
    write_material_columns(mesh.getSchema().getArbGeomParams(), m.cnt.size(), kNames, 5, false);

    OXform lxf(top, "light_xf");
    XformSample ls;
    ls.setTranslation(V3d(0.0, 2.5, 0.0));
    ls.setXRotation(90.0);
    ls.setScale(V3d(0.5, 0.5, 1.0));
    lxf.getSchema().set(ls);
    MeshSpec lm = grid_mesh(1, 1, 0.0f, false);
    OPolyMesh light = write_mesh(lxf, "light", lm);
    {
        OCompoundProperty arb = light.getSchema().getArbGeomParams();
        std::vector<std::string> vals = {"Lambertian"};
        std::vector<uint32_t> which(lm.cnt.size(), 0u);
        OStringGeomParam mat(arb, "material", true, kUniformScope, 1);
        mat.set(OStringGeomParam::Sample(StringArraySample(vals), UInt32ArraySample(which), kUniformScope));
        std::vector<C3f> le(lm.cnt.size(), C3f(12.0f, 11.0f, 9.0f));
        OC3fGeomParam pLe(arb, "Le", false, kUniformScope, 1);
        pLe.set(OC3fGeomParam::Sample(C3fArraySample(le), kUniformScope));
        std::vector<int32_t> back(lm.cnt.size(), 1);
        OInt32GeomParam pb(arb, "BackEmission", false, kUniformScope, 1);
        pb.set(OInt32GeomParam::Sample(Int32ArraySample(back), kUniformScope));
    }

    OXform pxf(top, "balls_xf");
    XformSample ident;
    pxf.getSchema().set(ident);
    OPoints pts(pxf, "balls");
    std::vector<V3f> pp;
    std::vector<uint64_t> ids;
    std::vector<float> rad;
    std::vector<C3f> cd;
    for (int i = 0; i < 5; ++i) {
        pp.push_back(V3f(-1.6f + 0.8f * i, 0.35f, 0.2f * (i % 2)));
        ids.push_back((uint64_t)i);
        rad.push_back(0.3f);
        cd.push_back(C3f(rnd(), rnd(), rnd()));
    }
    pts.getSchema().set(OPointsSchema::Sample(P3fArraySample(pp), UInt64ArraySample(ids)));
    OCompoundProperty parb = pts.getSchema().getArbGeomParams();
    OFloatGeomParam pscale(parb, "pscale", false, kVaryingScope, 1);
    pscale.set(OFloatGeomParam::Sample(FloatArraySample(rad), kVaryingScope));
    OC3fGeomParam pcd(parb, "Cd", false, kVaryingScope, 1);
    pcd.set(OC3fGeomParam::Sample(C3fArraySample(cd), kVaryingScope));

    OXform cxf(top, "cam_xf");
    XformSample cxs;
    cxs.setTranslation(V3d(0.0, 1.2, 4.5));
    cxs.setXRotation(-12.0);
    cxf.getSchema().set(cxs);
    OCamera cam(cxf, "cam");
    CameraSample csmp;
    csmp.setFocalLength(30.0);
    csmp.setHorizontalAperture(3.6);
    csmp.setVerticalAperture(2.7);
    csmp.setFocusDistance(4.5);
    csmp.setFStop(16.0);
    cam.getSchema().set(csmp);
    OCompoundProperty up = cam.getSchema().getUserProperties();
    OFloatProperty resx(up, "resx"), resy(up, "resy");
    resx.set(96.0f);
    resy.set(72.0f);
}

// Three frames: a transform and vertex positions sampled per frame (a
// 1/24 s time sampling), constant topology and material columns.
void write_anim(const char* path) {
    g_state = 99u;
    OArchive archive(Alembic::AbcCoreOgawa::WriteArchive(), path);
    OObject top = archive.getTop();
    TimeSamplingPtr ts(new TimeSampling(1.0 / 24.0, 0.0));
    const uint32_t tsi = archive.addTimeSampling(*ts);
    OXform xf(top, "anim_xf", tsi);
    OPolyMesh mesh(xf, "anim_mesh", tsi);
    MeshSpec m = grid_mesh(2, 2, 0.0f, false);
    static const char* const kNames[] = {"Lambertian", "Ward"};
    for (int f = 0; f < 3; ++f) {
        XformSample xs;
        xs.setTranslation(V3d(0.25 * f, 0.0, -0.5 * f));
        xs.setZRotation(10.0 * f);
        xf.getSchema().set(xs);
        std::vector<V3f> P = m.P;
        for (auto& p : P) p.z += 0.1f * (float)f;
        if (f == 0) {
            OPolyMeshSchema::Sample s(P3fArraySample(P), Int32ArraySample(m.idx), Int32ArraySample(m.cnt));
            mesh.getSchema().set(s);
        } else {
            OPolyMeshSchema::Sample s((P3fArraySample(P)));
            mesh.getSchema().set(s);
        }
    }
    write_material_columns(mesh.getSchema().getArbGeomParams(), m.cnt.size(), kNames, 2, false);
}

// A mesh whose "material" names a class the reference does not register.
void write_badmat(const char* path) {
    OArchive archive(Alembic::AbcCoreOgawa::WriteArchive(), path);
    OObject top = archive.getTop();
    OXform xf(top, "bad_xf");
    XformSample ident;
    xf.getSchema().set(ident);
    MeshSpec m = grid_mesh(1, 1, 0.0f, false);
    static const char* const kNames[] = {"Lambertian", "Glass"};
    write_material_columns(write_mesh(xf, "bad", m).getSchema().getArbGeomParams(), m.cnt.size(), kNames, 2, false);
}

// ---------------------------------------------------------------- dumping
void pf(float v) {
    if (std::isfinite(v))
        std::printf("%.9g", (double)v);
    else
        std::printf("\"%s\"", std::isnan(v) ? "nan" : (v > 0 ? "inf" : "-inf"));
}
void pstr(const std::string& s) {
    std::putchar('"');
    for (unsigned char c : s) {
        if (c == '"' || c == '\\')
            std::printf("\\%c", c);
        else if (c < 0x20)
            std::printf("\\u%04x", c);
        else
            std::putchar(c);
    }
    std::putchar('"');
}
void pmat(const houdini_alembic::Matrix4x4f& m) {
    std::printf("[");
    for (int i = 0; i < 16; ++i) {
        if (i) std::printf(",");
        pf(m.value[i]);
    }
    std::printf("]");
}
void pvec(const houdini_alembic::Vector3f& v) {
    std::printf("[");
    pf(v.x);
    std::printf(",");
    pf(v.y);
    std::printf(",");
    pf(v.z);
    std::printf("]");
}

void dump_sheet(const houdini_alembic::AttributeSpreadSheet& s) {
    using namespace houdini_alembic;
    std::printf("[");
    for (size_t c = 0; c < s.sheet.size(); ++c) {
        const auto& a = s.sheet[c];
        if (c) std::printf(",");
        std::printf("{\"key\":");
        pstr(a.key);
        const AttributeColumn* col = a.column.get();
        std::printf(",\"type\":\"%s\",\"rows\":%u,\"values\":[", attributeTypeString(col->attributeType()),
                    col->rowCount());
        for (uint32_t r = 0; r < col->rowCount(); ++r) {
            if (r) std::printf(",");
            switch (col->attributeType()) {
                case AttributeType_Int:
                    std::printf("%d", static_cast<const AttributeIntColumn*>(col)->get(r));
                    break;
                case AttributeType_Float:
                    pf(static_cast<const AttributeFloatColumn*>(col)->get(r));
                    break;
                case AttributeType_String:
                    pstr(static_cast<const AttributeStringColumn*>(col)->get(r));
                    break;
                default: {
                    float v[4] = {0, 0, 0, 0};
                    int n = 2;
                    if (col->attributeType() == AttributeType_Vector2) {
                        static_cast<const AttributeVector2Column*>(col)->get(r, v);
                    } else if (col->attributeType() == AttributeType_Vector3) {
                        static_cast<const AttributeVector3Column*>(col)->get(r, v);
                        n = 3;
                    } else {
                        static_cast<const AttributeVector4Column*>(col)->get(r, v);
                        n = 4;
                    }
                    std::printf("[");
                    for (int k = 0; k < n; ++k) {
                        if (k) std::printf(",");
                        pf(v[k]);
                    }
                    std::printf("]");
                }
            }
        }
        std::printf("]}");
    }
    std::printf("]");
}

int dump(const char* path, unsigned frame) {
    using namespace houdini_alembic;
    AlembicStorage storage;
    std::string err;
    if (!storage.open(path, err)) {
        std::fprintf(stderr, "open failed: %s\n", err.c_str());
        return 1;
    }
    auto scene = storage.read(frame, err);
    if (!scene) {
        std::fprintf(stderr, "read failed: %s\n", err.c_str());
        return 1;
    }
    std::printf("{\"frame_count\":%u,\"objects\":[", storage.frameCount());
    for (size_t i = 0; i < scene->objects.size(); ++i) {
        const SceneObjectPointer& o = scene->objects[i];
        if (i) std::printf(",\n");
        static const char* kTypes[] = {"PolygonMesh", "Point", "Curve", "Camera"};
        std::printf("{\"type\":\"%s\",\"name\":", kTypes[o->type()]);
        pstr(o->name);
        std::printf(",\"visible\":%s,\"combined\":", o->visible ? "true" : "false");
        pmat(o->combinedXforms);
        std::printf(",\"xforms\":[");
        for (size_t k = 0; k < o->xforms.size(); ++k) {
            if (k) std::printf(",");
            pmat(o->xforms[k]);
        }
        std::printf("]");
        if (auto m = o.as_polygonMesh()) {
            std::printf(",\"faceCounts\":[");
            for (size_t k = 0; k < m->faceCounts.size(); ++k) std::printf("%s%u", k ? "," : "", m->faceCounts[k]);
            std::printf("],\"indices\":[");
            for (size_t k = 0; k < m->indices.size(); ++k) std::printf("%s%u", k ? "," : "", m->indices[k]);
            std::printf("],\"P\":[");
            for (size_t k = 0; k < m->P.size(); ++k) {
                if (k) std::printf(",");
                pvec(m->P[k]);
            }
            std::printf("],\"points\":");
            dump_sheet(m->points);
            std::printf(",\"vertices\":");
            dump_sheet(m->vertices);
            std::printf(",\"primitives\":");
            dump_sheet(m->primitives);
        } else if (auto p = o.as_point()) {
            std::printf(",\"pointIds\":[");
            for (size_t k = 0; k < p->pointIds.size(); ++k)
                std::printf("%s%llu", k ? "," : "", (unsigned long long)p->pointIds[k]);
            std::printf("],\"P\":[");
            for (size_t k = 0; k < p->P.size(); ++k) {
                if (k) std::printf(",");
                pvec(p->P[k]);
            }
            std::printf("],\"points\":");
            dump_sheet(p->points);
        } else if (auto c = o.as_camera()) {
            std::printf(",\"eye\":");
            pvec(c->eye);
            std::printf(",\"lookat\":");
            pvec(c->lookat);
            std::printf(",\"up\":");
            pvec(c->up);
            std::printf(",\"down\":");
            pvec(c->down);
            std::printf(",\"forward\":");
            pvec(c->forward);
            std::printf(",\"back\":");
            pvec(c->back);
            std::printf(",\"left\":");
            pvec(c->left);
            std::printf(",\"right\":");
            pvec(c->right);
            std::printf(",\"resolution_x\":%d,\"resolution_y\":%d", c->resolution_x, c->resolution_y);
            const float f[] = {c->focalLength_mm, c->aperture_horizontal_mm, c->aperture_vertical_mm,
                               c->nearClip, c->farClip, c->focusDistance, c->f_stop, c->fov_horizontal_degree,
                               c->fov_vertical_degree, c->lensRadius, c->objectPlaneWidth, c->objectPlaneHeight};
            const char* names[] = {"focalLength_mm", "aperture_horizontal_mm", "aperture_vertical_mm", "nearClip",
                                   "farClip", "focusDistance", "f_stop", "fov_horizontal_degree",
                                   "fov_vertical_degree", "lensRadius", "objectPlaneWidth", "objectPlaneHeight"};
            for (int k = 0; k < 12; ++k) {
                std::printf(",\"%s\":", names[k]);
                pf(f[k]);
            }
        }
        std::printf("}");
    }
    std::printf("]}\n");
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc >= 4 && std::strcmp(argv[1], "write") == 0) {
        try {
            if (std::strcmp(argv[3], "basic") == 0)
                write_basic(argv[2]);
            else if (std::strcmp(argv[3], "render") == 0)
                write_render(argv[2]);
            else if (std::strcmp(argv[3], "anim") == 0)
                write_anim(argv[2]);
            else if (std::strcmp(argv[3], "badmat") == 0)
                write_badmat(argv[2]);
            else {
                std::fprintf(stderr, "unknown scene %s\n", argv[3]);
                return 2;
            }
        } catch (std::exception& e) {
            std::fprintf(stderr, "write failed: %s\n", e.what());
            return 1;
        }
        return 0;
    }
    if (argc >= 3 && std::strcmp(argv[1], "dump") == 0) return dump(argv[2], argc >= 4 ? (unsigned)std::atoi(argv[3]) : 0u);
    std::fprintf(stderr, "usage: abc_tool write <out.abc> basic|render|anim|badmat | abc_tool dump <in.abc> [frame]\n");
    return 2;
}
