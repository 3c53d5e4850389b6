/* ref_assets.c — test infrastructure only: the checker for the asset loaders.
 *
 * Restates the data extraction of the reference's scene loaders,
 * core/assets/asset_loader.cpp:367-611 (glTF through cgltf) and :613-920 (FBX
 * through ufbx), on top of the very libraries the reference vendors
 * (extern/cgltf/cgltf.h and extern/ufbx/ufbx.c, compiled from the reference
 * checkout by oracle/build_ref.sh; nothing of them is copied here).  Instead of
 * calling the renderer it writes what the loader would hand it to a flat dump
 * that tests/test_gltf.py and tests/test_fbx.py (through tests/ref_assets.py)
 * compare with wavefrontpathtracing_gb300.gltf
 * and wavefrontpathtracing_gb300.fbx.
 *
 * Where the reference is undefined this restatement takes the defined choice
 * the Python loaders document (each marked "defined here"):
 *   glTF: ret.nodes is indexed by the glTF node index although it only holds
 *         the nodes with a mesh (asset_loader.cpp:580), and a node's mesh
 *         indices are primitive indices within its own glTF mesh
 *         (asset_loader.cpp:600); here every node with a mesh contributes one
 *         instance per primitive of its mesh, in node order, indexing the
 *         global primitive list.
 *   FBX:  the running mesh-part counter advances once per part per instance
 *         (asset_loader.cpp:896-905), so a mesh used by several nodes hands
 *         the later nodes other meshes' parts, and parts without triangles are
 *         counted there but skipped as meshes (:785); a mesh without materials
 *         reads materials[0] of an empty list (:903).  Here each instance gets
 *         its own mesh's non-empty parts and material -1 (the default) when
 *         the mesh has none.
 *
 * Dump (little endian):
 *   u32 'WFAD', u32 1
 *   u32 materials; each: f32 base[4], metallic, roughness, emissive[3],
 *       emissive_strength; then for base colour, normal, metallic-roughness,
 *       emissive: i32 glTF image index (-1 none) and a string (FBX texture
 *       relative filename, "" none): u32 length + bytes
 *   u32 meshes; each: u32 vertices, vertices x 8 f32 (position, normal, uv),
 *       u32 indices, indices x u32
 *   u32 instances; each: u32 mesh, i32 material (-1 none), f32[16]
 *       node_to_world (glm column-major)
 */
#define CGLTF_IMPLEMENTATION
#include "cgltf/cgltf.h"
#include "ufbx/ufbx.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    float pos[3], normal[3], uv[2];
} dump_vertex;

typedef struct {
    FILE* f;
} out_t;

static void w_u32(out_t* o, uint32_t v) { fwrite(&v, 4, 1, o->f); }
static void w_i32(out_t* o, int32_t v) { fwrite(&v, 4, 1, o->f); }
static void w_f32(out_t* o, float v) { fwrite(&v, 4, 1, o->f); }
static void w_str(out_t* o, const char* s, size_t n) {
    w_u32(o, (uint32_t)n);
    if (n) fwrite(s, 1, n, o->f);
}

typedef struct {
    float base[4], metallic, roughness, emissive[3], strength;
    int32_t image[4];
    const char* name[4];
    size_t name_len[4];
} dump_material;

static void w_material(out_t* o, const dump_material* m) {
    for (int k = 0; k < 4; ++k) w_f32(o, m->base[k]);
    w_f32(o, m->metallic);
    w_f32(o, m->roughness);
    for (int k = 0; k < 3; ++k) w_f32(o, m->emissive[k]);
    w_f32(o, m->strength);
    for (int k = 0; k < 4; ++k) {
        w_i32(o, m->image[k]);
        w_str(o, m->name[k] ? m->name[k] : "", m->name[k] ? m->name_len[k] : 0);
    }
}

/* ------------------------------------------------------------------ glTF */

static int32_t gltf_image_of(const cgltf_data* d, const cgltf_texture_view* v) {
    if (!v->texture || !v->texture->image) return -1;
    return (int32_t)(v->texture->image - d->images);
}

static int dump_gltf(const char* path, out_t* o) {
    cgltf_options opt;
    memset(&opt, 0, sizeof(opt));
    cgltf_data* d = NULL;
    if (cgltf_parse_file(&opt, path, &d) != cgltf_result_success) return 2;
    if (cgltf_load_buffers(&opt, d, path) != cgltf_result_success) {
        cgltf_free(d);
        return 3;
    }
    /* materials: asset_loader.cpp:411-471 */
    w_u32(o, (uint32_t)d->materials_count);
    for (cgltf_size i = 0; i < d->materials_count; ++i) {
        const cgltf_material* g = &d->materials[i];
        dump_material m;
        memset(&m, 0, sizeof(m));
        m.base[0] = m.base[1] = m.base[2] = m.base[3] = 1.0f;
        m.metallic = 1.0f;
        m.roughness = 1.0f;
        for (int k = 0; k < 4; ++k) m.image[k] = -1;
        if (g->has_pbr_metallic_roughness) {
            memcpy(m.base, g->pbr_metallic_roughness.base_color_factor, 16);
            m.metallic = g->pbr_metallic_roughness.metallic_factor;
            m.roughness = g->pbr_metallic_roughness.roughness_factor;
            memcpy(m.emissive, g->emissive_factor, 12);
            m.strength = g->emissive_strength.emissive_strength;
            m.image[0] = gltf_image_of(d, &g->pbr_metallic_roughness.base_color_texture);
            m.image[1] = gltf_image_of(d, &g->normal_texture);
            m.image[2] = gltf_image_of(d, &g->pbr_metallic_roughness.metallic_roughness_texture);
            m.image[3] = gltf_image_of(d, &g->emissive_texture);
        }
        w_material(o, &m);
    }
    /* meshes, one per primitive: asset_loader.cpp:476-565 (accessors read
     * through cgltf_accessor_read_* so strided views and 8-bit indices are
     * handled; the reference memcpy's tightly packed data) */
    cgltf_size prims = 0;
    for (cgltf_size i = 0; i < d->meshes_count; ++i) prims += d->meshes[i].primitives_count;
    w_u32(o, (uint32_t)prims);
    for (cgltf_size i = 0; i < d->meshes_count; ++i) {
        for (cgltf_size p = 0; p < d->meshes[i].primitives_count; ++p) {
            const cgltf_primitive* pr = &d->meshes[i].primitives[p];
            const cgltf_accessor *pos = NULL, *nrm = NULL, *uv = NULL;
            for (cgltf_size a = 0; a < pr->attributes_count; ++a) {
                const cgltf_attribute* at = &pr->attributes[a];
                if (at->type == cgltf_attribute_type_position) pos = at->data;
                if (at->type == cgltf_attribute_type_normal) nrm = at->data;
                if (at->type == cgltf_attribute_type_texcoord && at->index == 0) uv = at->data;
            }
            if (!pos || !nrm || !uv) {
                cgltf_free(d);
                return 4;
            }
            w_u32(o, (uint32_t)pos->count);
            for (cgltf_size v = 0; v < pos->count; ++v) {
                dump_vertex dv;
                memset(&dv, 0, sizeof(dv));
                cgltf_accessor_read_float(pos, v, dv.pos, 3);
                cgltf_accessor_read_float(nrm, v, dv.normal, 3);
                cgltf_accessor_read_float(uv, v, dv.uv, 2);
                fwrite(&dv, sizeof(dv), 1, o->f);
            }
            if (pr->indices) {
                w_u32(o, (uint32_t)pr->indices->count);
                for (cgltf_size k = 0; k < pr->indices->count; ++k)
                    w_u32(o, (uint32_t)cgltf_accessor_read_index(pr->indices, k));
            } else {
                w_u32(o, (uint32_t)pos->count);
                for (cgltf_size k = 0; k < pos->count; ++k) w_u32(o, (uint32_t)k);
            }
        }
    }
    /* nodes with a mesh -> instances: asset_loader.cpp:569-608 (defined here:
     * global primitive indices, node order) */
    uint32_t count = 0;
    for (cgltf_size n = 0; n < d->nodes_count; ++n)
        if (d->nodes[n].mesh) count += (uint32_t)d->nodes[n].mesh->primitives_count;
    w_u32(o, count);
    for (cgltf_size n = 0; n < d->nodes_count; ++n) {
        const cgltf_node* nd = &d->nodes[n];
        if (!nd->mesh) continue;
        cgltf_float world[16];
        cgltf_node_transform_world(nd, world);
        uint32_t first = 0;
        for (cgltf_size i = 0; i < (cgltf_size)(nd->mesh - d->meshes); ++i) first += (uint32_t)d->meshes[i].primitives_count;
        for (cgltf_size p = 0; p < nd->mesh->primitives_count; ++p) {
            w_u32(o, first + (uint32_t)p);
            const cgltf_material* mt = nd->mesh->primitives[p].material;
            w_i32(o, mt ? (int32_t)(mt - d->materials) : -1);
            for (int k = 0; k < 16; ++k) w_f32(o, world[k]);
        }
    }
    cgltf_free(d);
    return 0;
}

/* ------------------------------------------------------------------ FBX */

static void fbx_texture_name(const ufbx_texture* t, const char** s, size_t* n) {
    *s = NULL;
    *n = 0;
    if (!t) return;
    *s = t->relative_filename.data;
    *n = t->relative_filename.length;
}

static int dump_fbx(const char* path, out_t* o) {
    /* load options: asset_loader.cpp:658-684 */
    ufbx_load_opts opts;
    memset(&opts, 0, sizeof(opts));
    opts.file_format = UFBX_FILE_FORMAT_FBX;
    opts.target_unit_meters = 1.0f;
    opts.generate_missing_normals = true;
    opts.normalize_normals = true;
    opts.normalize_tangents = true;
    opts.target_axes.right = UFBX_COORDINATE_AXIS_POSITIVE_X;
    opts.target_axes.up = UFBX_COORDINATE_AXIS_POSITIVE_Y;
    opts.target_axes.front = UFBX_COORDINATE_AXIS_POSITIVE_Z;
    opts.space_conversion = UFBX_SPACE_CONVERSION_MODIFY_GEOMETRY;
    ufbx_error err;
    ufbx_scene* sc = ufbx_load_file(path, &opts, &err);
    if (!sc) return 2;

    /* materials: asset_loader.cpp:688-754 */
    w_u32(o, (uint32_t)sc->materials.count);
    for (size_t i = 0; i < sc->materials.count; ++i) {
        const ufbx_material* fm = sc->materials.data[i];
        dump_material m;
        memset(&m, 0, sizeof(m));
        for (int k = 0; k < 4; ++k) m.image[k] = -1;
        m.base[0] = m.base[1] = m.base[2] = 0.8f;
        m.base[3] = 1.0f;
        m.metallic = 0.0f;
        m.roughness = 0.5f;
        if (fm->features.pbr.enabled || fm->features.specular.enabled) {
            m.base[0] = m.base[1] = m.base[2] = m.base[3] = 1.0f;
            m.metallic = 1.0f;
            m.roughness = 1.0f;
            if (fm->pbr.base_color.texture_enabled) fbx_texture_name(fm->pbr.base_color.texture, &m.name[0], &m.name_len[0]);
            if (fm->pbr.normal_map.texture_enabled) fbx_texture_name(fm->pbr.normal_map.texture, &m.name[1], &m.name_len[1]);
            if (fm->pbr.metalness.texture_enabled || fm->pbr.roughness.texture_enabled) {
                const ufbx_texture* tm = fm->pbr.metalness.texture;
                const ufbx_texture* tr = fm->pbr.roughness.texture;
                if (tm && tr && tm == tr) fbx_texture_name(tm, &m.name[2], &m.name_len[2]);
            } else if (fm->pbr.specular_color.texture_enabled) {
                fbx_texture_name(fm->pbr.specular_color.texture, &m.name[2], &m.name_len[2]);
            }
            if (fm->pbr.emission_color.texture_enabled)
                fbx_texture_name(fm->pbr.emission_color.texture, &m.name[3], &m.name_len[3]);
        }
        w_material(o, &m);
    }

    /* meshes, one per non-empty material part of an instanced mesh:
     * asset_loader.cpp:758-843 */
    uint32_t nmesh = 0;
    size_t max_tris = 0;
    for (size_t i = 0; i < sc->meshes.count; ++i) {
        const ufbx_mesh* fm = sc->meshes.data[i];
        if (fm->instances.count == 0) continue;
        for (size_t p = 0; p < fm->material_parts.count; ++p) {
            if (fm->material_parts.data[p].num_triangles == 0) continue;
            nmesh++;
            if (fm->material_parts.data[p].num_triangles > max_tris) max_tris = fm->material_parts.data[p].num_triangles;
        }
    }
    w_u32(o, nmesh);
    uint32_t* first_part = (uint32_t*)calloc(sc->meshes.count + 1, sizeof(uint32_t));
    dump_vertex* verts = (dump_vertex*)calloc(max_tris * 3 + 1, sizeof(dump_vertex));
    uint32_t* idx = (uint32_t*)calloc(max_tris * 3 + 1, sizeof(uint32_t));
    uint32_t next = 0;
    for (size_t i = 0; i < sc->meshes.count; ++i) {
        const ufbx_mesh* fm = sc->meshes.data[i];
        first_part[i] = next;
        if (fm->instances.count == 0 || fm->material_parts.count == 0) continue;
        if (!fm->vertex_position.exists || !fm->vertex_normal.exists || !fm->vertex_uv.exists) {
            free(first_part); free(verts); free(idx);
            ufbx_free_scene(sc);
            return 4;
        }
        size_t ntri_idx = fm->max_face_triangles * 3;
        uint32_t* tri = (uint32_t*)calloc(ntri_idx + 1, sizeof(uint32_t));
        for (size_t p = 0; p < fm->material_parts.count; ++p) {
            const ufbx_mesh_part* part = &fm->material_parts.data[p];
            if (part->num_triangles == 0) continue;
            size_t n = 0;
            memset(verts, 0, (max_tris * 3 + 1) * sizeof(dump_vertex));
            for (size_t f = 0; f < part->num_faces; ++f) {
                ufbx_face face = fm->faces.data[part->face_indices.data[f]];
                uint32_t nt = ufbx_triangulate_face(tri, ntri_idx, fm, face);
                for (uint32_t k = 0; k < nt * 3; ++k) {
                    uint32_t c = tri[k];
                    ufbx_vec3 pp = ufbx_get_vertex_vec3(&fm->vertex_position, c);
                    ufbx_vec3 nn = ufbx_get_vertex_vec3(&fm->vertex_normal, c);
                    ufbx_vec2 tt = ufbx_get_vertex_vec2(&fm->vertex_uv, c);
                    verts[n].pos[0] = (float)pp.x; verts[n].pos[1] = (float)pp.y; verts[n].pos[2] = (float)pp.z;
                    verts[n].normal[0] = (float)nn.x; verts[n].normal[1] = (float)nn.y; verts[n].normal[2] = (float)nn.z;
                    verts[n].uv[0] = (float)tt.x;
                    verts[n].uv[1] = (float)(1.0f - tt.y);
                    n++;
                }
            }
            ufbx_vertex_stream stream;
            memset(&stream, 0, sizeof(stream));
            stream.data = verts;
            stream.vertex_count = n;
            stream.vertex_size = sizeof(dump_vertex);
            size_t nv = ufbx_generate_indices(&stream, 1, idx, n, NULL, NULL);
            w_u32(o, (uint32_t)nv);
            fwrite(verts, sizeof(dump_vertex), nv, o->f);
            w_u32(o, (uint32_t)n);
            fwrite(idx, 4, n, o->f);
            next++;
        }
        free(tri);
    }

    /* nodes: asset_loader.cpp:849-914 (defined here: each instance gets its
     * own mesh's parts) */
    uint32_t ninst = 0;
    for (size_t i = 0; i < sc->meshes.count; ++i) {
        const ufbx_mesh* fm = sc->meshes.data[i];
        if (fm->instances.count == 0 || fm->material_parts.count == 0) continue;
        uint32_t parts = 0;
        for (size_t p = 0; p < fm->material_parts.count; ++p) parts += fm->material_parts.data[p].num_triangles ? 1u : 0u;
        for (size_t k = 0; k < fm->instances.count; ++k)
            if (fm->instances.data[k]->visible) ninst += parts;
    }
    w_u32(o, ninst);
    for (size_t i = 0; i < sc->meshes.count; ++i) {
        const ufbx_mesh* fm = sc->meshes.data[i];
        if (fm->instances.count == 0 || fm->material_parts.count == 0) continue;
        for (size_t k = 0; k < fm->instances.count; ++k) {
            const ufbx_node* nd = fm->instances.data[k];
            if (!nd->visible) continue;
            const ufbx_matrix* M = &nd->node_to_world;
            const float cm[16] = {(float)M->m00, (float)M->m10, (float)M->m20, 0.0f,
                                  (float)M->m01, (float)M->m11, (float)M->m21, 0.0f,
                                  (float)M->m02, (float)M->m12, (float)M->m22, 0.0f,
                                  (float)M->m03, (float)M->m13, (float)M->m23, 1.0f};
            uint32_t m = first_part[i];
            for (size_t p = 0; p < fm->material_parts.count; ++p) {
                if (fm->material_parts.data[p].num_triangles == 0) continue;
                w_u32(o, m++);
                w_i32(o, p < fm->materials.count ? (int32_t)fm->materials.data[p]->typed_id : -1);
                for (int c = 0; c < 16; ++c) w_f32(o, cm[c]);
            }
        }
    }
    free(first_part); free(verts); free(idx);
    ufbx_free_scene(sc);
    return 0;
}

int ref_asset_dump(const char* in_path, const char* out_path) {
    const char* dot = strrchr(in_path, '.');
    if (!dot) return 1;
    out_t o;
    o.f = fopen(out_path, "wb");
    if (!o.f) return 1;
    w_u32(&o, 0x44414657u);   /* "WFAD" */
    w_u32(&o, 1u);
    int rc;
    if (strcmp(dot, ".gltf") == 0 || strcmp(dot, ".glb") == 0) rc = dump_gltf(in_path, &o);
    else if (strcmp(dot, ".fbx") == 0) rc = dump_fbx(in_path, &o);
    else rc = 1;
    fclose(o.f);
    return rc;
}
