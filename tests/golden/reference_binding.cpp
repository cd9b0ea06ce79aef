// The reference-side C++ a maintainer adds to bind the reference to this
// library: the render_multiThread replacement
// (src/render.cpp), the image loaders (src/material.cpp, src/component.cpp)
// and the model creation of MyConsole (src/myconsole.cpp:13-23).
// tests/test_library.py compiles this file against the reference's own
// headers (with the oracle's glm / assimp / libpng stand-ins) and
// include/rmn.h.
#include <mutex>
#include <thread>
#include <iostream>
#include <stdexcept>
#include "render.h"
#include "geometry.h"
#include "image.h"
#include "sampling.h"
#include "material.h"
#include "component.h"

// ---- src/render.cpp
#include <cstring>
#include "rmn.h"   // this repository's include/rmn.h; link with -lrmn

static_assert(sizeof(rmn_material) == 16 * sizeof(float), "ABI");

void render_multiThread(Model &model, const RenderArgs &args) {
    // 1. Model -> rmn_scene_desc. Faces hold their own vertices and pointers
    //    to VertexData, so emit three vertices per face.
    const int nt = (int)model.faces.size();
    std::vector<float> pos(9 * nt), nrm(9 * nt), uv(6 * nt);
    std::vector<int32_t> idx(3 * nt), first, mesh_mat;
    for (int f = 0; f < nt; ++f) {
        const Face &F = model.faces[f];
        for (int k = 0; k < 3; ++k) {
            for (int c = 0; c < 3; ++c) { pos[9*f + 3*k + c] = F.v[k][c]; nrm[9*f + 3*k + c] = F.data[k]->normal[c]; }
            uv[6*f + 2*k] = F.data[k]->uv.x; uv[6*f + 2*k + 1] = F.data[k]->uv.y;
            idx[3*f + k] = 3*f + k;
        }
        int m = F.material->id;                 // one mesh per run of equal materials
        if (mesh_mat.empty() || mesh_mat.back() != m) { first.push_back(f); mesh_mat.push_back(m); }
    }
    first.push_back(nt);
    // Materials: every texture the loader filled goes over as it is (level 0;
    // librmn builds the mip chain as ImageData::generateMipmaps does); an
    // empty slot keeps the reference's default (white diffuse, no emission,
    // Material::roughness, metallic 0), i.e. no constant texel.
    std::vector<rmn_material> mats(model.materials.size());
    std::vector<rmn_texture> texs;
    std::vector<int32_t> mat_tex(4 * mats.size(), -1);
    const int slot[4] = {aiTextureType_DIFFUSE, aiTextureType_SPECULAR, aiTextureType_EMISSIVE,
                         aiTextureType_NORMALS};              // RMN_TEX_DIFFUSE .. RMN_TEX_NORMALS
    for (size_t i = 0; i < mats.size(); ++i) {
        const Material &M = model.materials[i];
        for (int k = 0; k < 4; ++k) {
            const ImageData &T = M.texture[slot[k]];
            if (T.empty()) continue;
            if (T.channels != 4) { std::cerr << "texture is not RGBA8" << std::endl; return; }
            mat_tex[4 * i + k] = (int32_t)texs.size();
            texs.push_back(rmn_texture{T.width, T.height, T.channels, T.data[0].data()});
        }
        mats[i] = rmn_material{{1.0f, 1.0f, 1.0f}, 0.0f, {0.0f, 0.0f, 0.0f}, 0.0f,
                               M.roughness, 0.0f, 0.0f, M.opacity, M.ior,
                               {M.transmittingColor.x, M.transmittingColor.y, M.transmittingColor.z}};
    }
    // SkyBox::data is premultiplied by the texel solid angle; hand over the
    // radiance it was loaded with (SkyBox::get divides the same factor out).
    std::vector<float> sky;
    if (!model.skyMap.empty()) {
        sky.resize(3 * model.skyMap.data.size());
        for (int v = 0; v < model.skyMap.height; ++v)
            for (int u = 0; u < model.skyMap.width; ++u) {
                int i = v * model.skyMap.width + u;
                float phi = PI * (float(v) + 0.5f) / float(model.skyMap.height);
                float area = sin(phi) * 2.0f * PI / float(model.skyMap.width * model.skyMap.height);
                for (int c = 0; c < 3; ++c) sky[3*i + c] = model.skyMap.data[i][c] / area;
            }
    }
    rmn_scene_desc desc{3 * nt, pos.data(), nrm.data(), uv.data(), nt, idx.data(),
                        (int32_t)mesh_mat.size(), first.data(), mesh_mat.data(),
                        (int32_t)mats.size(), mats.data(),
                        model.skyMap.width, model.skyMap.height, sky.empty() ? nullptr : sky.data(),
                        (int32_t)texs.size(), texs.data(), mat_tex.data()};
    rmn_scene *scene = nullptr;
    if (rmn_scene_create(&desc, &scene) != RMN_OK) { std::cerr << rmn_last_error() << std::endl; return; }

    // 2. Render into the Photo's own buffers (host memory; staged by librmn).
    Photo photo(args.width, args.height);
    photo.exposure = args.exposure;
    const size_t npx = (size_t)args.width * args.height;
    std::vector<float> gbuf(npx * RMN_GBUFFER_FLOATS);
    rmn_render_args ra{};
    for (int c = 0; c < 3; ++c) {
        ra.position[c] = args.position[c]; ra.direction[c] = args.direction[c];
        ra.up[c] = args.up[c]; ra.right[c] = args.right[c];
    }
    ra.accuracy = args.accuracy; ra.focus = args.focus; ra.CoC = args.CoC;
    ra.exposure = args.exposure; ra.P_Direct = args.P_Direct;
    ra.width = args.width; ra.height = args.height; ra.spp = args.spp; ra.threads = args.threads;
    ra.max_depth = 16; ra.seed = 1;
    // RadianceData is {vec3 radiance; float Var;} = 4 floats, as rmn_image expects.
    rmn_image img{(float*)photo.radiance_Dd, (float*)photo.radiance_Ds,
                  (float*)photo.radiance_Id, (float*)photo.radiance_Is, gbuf.data(),
                  nullptr /* dropped: only rmn_adjoint needs it */};
    if (rmn_render(scene, &ra, &img, nullptr) != RMN_OK) std::cerr << rmn_last_error() << std::endl;
    for (size_t i = 0; i < npx; ++i) {         // G-buffer back into HitInfo for the exports
        const float *g = &gbuf[i * RMN_GBUFFER_FLOATS];
        HitInfo &h = photo.Gbuffer[i];
        h.baseColor = vec3(g[0], g[1], g[2]); h.emission = vec3(g[3], g[4], g[5]);
        h.position = vec3(g[6], g[7], g[8]);  h.shapeNormal = vec3(g[9], g[10], g[11]);
        h.surfaceNormal = vec3(g[12], g[13], g[14]);
        h.roughness = g[15]; h.metallic = g[16]; h.opacity = g[17]; h.eta = g[18]; h.id = (int)g[19];
        h.entering = g[20] != 0.0f;
    }
    rmn_scene_destroy(scene);

    // 3. Exports: on the GPU, all of src/render.cpp:641-674 in one call; each
    //    image then goes through Photo::save unchanged.
    {
        rmn_post_args pa{args.width, args.height, args.exposure, args.focus, args.CoC,
                         {args.position.x, args.position.y, args.position.z}};
        std::vector<float> rgb((size_t)(RMN_EXPORTS + RMN_EXPORTS_DOF) * 3 * npx);
        int32_t count = 0;
        if (rmn_export_set(&img, &pa, rgb.data(), &count, nullptr) != RMN_OK) std::cerr << rmn_last_error() << std::endl;
        for (int k = 0; k < count; ++k) {
            std::memcpy(photo.pixelarray, &rgb[(size_t)k * 3 * npx], 3 * npx * sizeof(float));
            photo.save((args.savePath + "(" + rmn_export_tag(k) + ").png").c_str());
        }
        return;
    }
    // (or exactly as before on the CPU, src/render.cpp:635-674:)
    auto exportImage = [&](const std::string &tag, int shadeOptions) {
        photo.postProcessing(shadeOptions);
        photo.save((args.savePath + "(" + tag + ").png").c_str());
    };
    exportImage("Raw", Photo::Full);
    exportImage("Raw_FXAA", Photo::Full | Photo::DoFXAA);
    // ... the remaining exports of src/render.cpp:641-674 unchanged
}

// ---- src/material.cpp, src/component.cpp
// src/material.cpp
static bool rmnLoad(ImageData &img, const std::string &file, int32_t kind) {
    rmn_image_desc d;
    if (rmn_image_load(file.c_str(), kind, &d, nullptr, 0) != RMN_OK) {
        std::cerr << rmn_last_error() << std::endl;
        return false;
    }
    img.data[0].resize((size_t)d.width * d.height * d.channels);
    if (rmn_image_load(file.c_str(), kind, &d, img.data[0].data(), img.data[0].size()) != RMN_OK) return false;
    img.width = d.width;
    img.height = d.height;
    img.channels = d.channels;   // PNG: 3 (the reference leaves it unset)
    return true;
}
bool Material::loadImageFromPNG(ImageData &img, const std::string &f) {
    if (!rmnLoad(img, f, RMN_IMAGE_PNG)) throw std::runtime_error("Error during PNG reading");
    return true;
}
bool Material::loadImageFromDDS(ImageData &img, const std::string &f) { return rmnLoad(img, f, RMN_IMAGE_DDS); }

// src/component.cpp
void SkyBox::load(const std::string &filename) {
    rmn_image_desc d;
    if (rmn_image_load(filename.c_str(), RMN_IMAGE_HDR, &d, nullptr, 0) != RMN_OK) return;
    std::vector<float> buf((size_t)d.width * d.height * 3);
    if (rmn_image_load(filename.c_str(), RMN_IMAGE_HDR, &d, buf.data(), buf.size() * sizeof(float)) != RMN_OK) return;
    width = d.width;
    height = d.height;
    for (size_t i = 0; i < buf.size() / 3; i++) data.emplace_back(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]);
    Init();
}

// ---- src/myconsole.cpp: create a model
void create_model(const std::string &folder, const std::string &name, const std::string &sky) {
rmn_model *m = nullptr;
if (rmn_model_read(folder.c_str(), name.c_str(), sky.c_str(), &m) != RMN_OK) {
    std::cerr << "Error loading model: " << rmn_last_error() << std::endl;
    return;
}
rmn_scene_desc d;
rmn_model_desc(m, &d);
rmn_scene *scene = nullptr;
rmn_scene_create(&d, &scene);   // BVH, light objects, sky tables, mip chains
rmn_model_free(m);              // the scene holds its own copies
}
