/*
 * agb.h - C ABI of the GB300 path-tracing backend for Aurora.
 *
 * This is the boundary between Aurora's C++ renderer interfaces (IRenderer / IScene / IMaterial /
 * IRenderBuffer, Libraries/Aurora/API/Aurora/Aurora.h:714-1226) and the sm_103a CUDA kernels.  The
 * reference has no such boundary: its HGI backend calls Vulkan ray tracing through USD Hgi.  Each
 * entry point below names the reference call it replaces.  Only plain C types cross it: no C++,
 * no CUDA or torch types.  Every function returns an agb_status (0 = success, negative = error);
 * agb_last_error() gives the message of the last failure on the calling thread.
 *
 * Pointers documented as "host" are read or written by the call itself (the call copies them);
 * "device" pointers must be CUDA device (or managed) memory on the context's GPU.
 */
#ifndef AGB_H
#define AGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define AGB_API __declspec(dllexport)
#else
#define AGB_API __attribute__((visibility("default")))
#endif

typedef int32_t agb_status;
enum
{
    AGB_OK              = 0,
    AGB_ERR_INVALID_ARG = -1,
    AGB_ERR_CUDA        = -2,
    AGB_ERR_OOM         = -3,
    AGB_ERR_TIMEOUT     = -4,
    AGB_ERR_NOT_READY   = -5,
    AGB_ERR_LIMIT       = -6
};

/* ------------------------------------------------------------------------------------------ */
/* Data layouts shared with the reference (byte-identical).                                   */
/* ------------------------------------------------------------------------------------------ */

/* Standard Surface material block, 400 bytes, std140 (Shaders/DefaultMaterialUniformBuffer.slang;
 * property order and defaults MaterialBase.cpp:28-167).  Uploaded per material by HGIMaterial
 * (HGI/HGIMaterial.cpp:23-60). */
typedef struct agb_material
{
    float base;
    float base_color[3];
    float diffuse_roughness;
    float metalness;
    float specular;
    int32_t _pad0;
    float specular_color[3];
    float specular_roughness;
    float specular_IOR;
    float specular_anisotropy;
    float specular_rotation;
    float transmission;
    float transmission_color[3];
    float subsurface;
    float subsurface_color[3];
    int32_t _pad1;
    float subsurface_radius[3];
    float subsurface_scale;
    float subsurface_anisotropy;
    float sheen;
    int32_t _pad2;
    int32_t _pad3;
    float sheen_color[3];
    float sheen_roughness;
    float coat;
    float coat_color[3];
    float coat_roughness;
    float coat_anisotropy;
    float coat_rotation;
    float coat_IOR;
    float coat_affect_color;
    float coat_affect_roughness;
    float emission;
    int32_t _pad4;
    float emission_color[3];
    int32_t _pad5;
    float opacity[3];
    int32_t thin_walled;
    int32_t has_base_color_image;
    float base_color_image_offset[2];
    int32_t _pad6;
    float base_color_image_scale[2];
    float base_color_image_pivot[2];
    float base_color_image_rotation;
    int32_t has_specular_roughness_image;
    float specular_roughness_image_offset[2];
    float specular_roughness_image_scale[2];
    float specular_roughness_image_pivot[2];
    float specular_roughness_image_rotation;
    int32_t has_emission_color_image;
    float emission_color_image_offset[2];
    float emission_color_image_scale[2];
    float emission_color_image_pivot[2];
    float emission_color_image_rotation;
    int32_t has_opacity_image;
    float opacity_image_offset[2];
    float opacity_image_scale[2];
    float opacity_image_pivot[2];
    float opacity_image_rotation;
    int32_t has_normal_image;
    float normal_image_offset[2];
    float normal_image_scale[2];
    float normal_image_pivot[2];
    float normal_image_rotation;
    int32_t _pad7;
    int32_t _pad8;
    int32_t _pad9;
} agb_material;

/* Texture slots of the built-in material, reference order (MaterialBase.cpp:97-103). */
enum
{
    AGB_TEX_BASE_COLOR         = 0,
    AGB_TEX_SPECULAR_ROUGHNESS = 1,
    AGB_TEX_OPACITY            = 2,
    AGB_TEX_NORMAL             = 3,
    AGB_TEX_EMISSION           = 4,
    AGB_TEX_SLOTS              = 5
};
/* Image index bound to each texture slot of one material; -1 = none. */
typedef struct agb_material_textures
{
    int32_t image[AGB_TEX_SLOTS];
} agb_material_textures;

/* One distant light (SceneBase.h:34-45; packed by HGIScene.cpp:118-132): direction already
 * negated (points toward the light), cos_radius = cos(0.5 * angular diameter). */
typedef struct agb_distant_light
{
    float color_and_intensity[4];
    float direction[3];
    float cos_radius;
} agb_distant_light;

/* Per-frame data, the reference's RendererBase::FrameData (RendererBase.h:136-241) byte for byte.
 * camera_inv_view holds the camera-to-world matrix stored row-major (the bytes of the reference's
 * transpose(inverse(view))): right = (m0,m4,m8), up = (m1,m5,m9), back = (m2,m6,m10),
 * eye = (m3,m7,m11).  view_size = (2 / P[0][0], 2 / P[1][1]). */
typedef struct agb_frame_data
{
    float camera_view_proj[16];
    float camera_view_proj_prev[16];
    float camera_inv_view[16];
    float camera_inv_view_prev[16];
    float view_size[2];
    float camera_jitter[2];
    float camera_jitter_prev[2];
    int32_t is_ortho_projection;
    float focal_distance;
    float lens_radius;
    float time_delta_ms;
    int32_t is_temporal_jitter_enabled;
    float scene_size;
    int32_t is_force_opaque_shadows_enabled;
    int32_t is_depth_ndc_enabled;
    int32_t is_diffuse_only_enabled;
    int32_t is_display_errors_enabled;
    int32_t is_denoising_enabled;
    int32_t is_denoising_aovs_enabled;
    int32_t trace_depth;
    float max_luminance;
    int32_t is_russian_roulette_enabled;
    int32_t russian_roulette_start_depth;
    int32_t is_path_regularization_enabled;
    float path_regularization_strength;
    float indirect_bounce_clamp_scale;
    float sky_view_z;
    float _padding1[2];
    agb_distant_light distant_lights[4];
    int32_t distant_light_count;
    int32_t _light_pad[3];
} agb_frame_data;

/* Environment constants, the reference's EnvironmentBase::EnvironmentData (EnvironmentBase.h:33-55)
 * byte for byte.  Matrices are stored row-major and applied to column vectors.  The luminance
 * integral is filled in by agb_environment_set when a light image is given. */
typedef struct agb_environment_data
{
    float light_top[3];
    float _padding1;
    float light_bottom[3];
    float light_tex_luminance_integral;
    float light_transform[16];
    float light_transform_inv[16];
    float background_top[3];
    float _padding3;
    float background_bottom[3];
    float _padding4;
    float background_transform[16];
    int32_t background_use_screen;
    int32_t has_light_tex;
    int32_t has_background_tex;
} agb_environment_data;

/* Alias-table entry (AliasMap.h:23-29). */
typedef struct agb_alias_entry
{
    uint32_t alias;
    float prob;
    float pdf;
    float _padding1;
} agb_alias_entry;

/* Ground plane (IGroundPlane, Aurora.h:780-806; the GPU constant data of PTGroundPlane.cpp:62-83):
 * an invisible plane that catches matte shadows of the environment light and a matte GGX
 * reflection, seen by camera rays only (GroundPlane.slang).  The side the normal points away from
 * is not rendered.  Defaults of a new ground plane (PTGroundPlane.cpp:42-51): enabled, position
 * 0, normal +Y, shadow opacity 1, shadow colour 0, reflection opacity 0.5, reflection colour 0.5,
 * reflection roughness 0.1.  The tangent frame is built from the normal. */
typedef struct agb_ground_plane
{
    int32_t enabled;
    float position[3];
    float normal[3];
    float shadow_opacity;
    float shadow_color[3];
    float reflection_opacity;
    float reflection_color[3];
    float reflection_roughness;
} agb_ground_plane;

/* ------------------------------------------------------------------------------------------ */
/* Scene description.                                                                          */
/* ------------------------------------------------------------------------------------------ */

/* One material layer of an instance (layer material + per-vertex UV set of the base mesh), the
 * DirectX layer data of PTScene.cpp:1051-1166 / GlobalBufferAccessors.slang:60-83.
 * texcoords: host, 2 floats per base-mesh vertex. */
typedef struct agb_layer
{
    int32_t material;
    int32_t _pad;
    const float* texcoords;
} agb_layer;

/* One instance (IScene::addInstancePointer, Aurora.h:1027-1029; HGIScene.cpp:383-397).
 * object_to_world: 3x4 row-major (rows of the reference's column-major mat4).  layers: host,
 * layer_count entries, outermost first as LayerDefinitions lists them. */
typedef struct agb_instance
{
    int32_t geometry;
    int32_t material;
    float object_to_world[12];
    int32_t layer_count;
    int32_t _pad;
    const agb_layer* layers;
} agb_instance;

/* Pixel formats of agb_image_create (Aurora.h:413-446 ImageFormat subset). */
enum
{
    AGB_FORMAT_RGBA8_UNORM = 0,
    AGB_FORMAT_RGBA32F     = 1,
    AGB_FORMAT_RGB32F      = 2
};

/* Accumulation modes of agb_render. */
enum
{
    /* FP32 running mean mix(prev, cur, 1/(n+1)) (HGI/Shaders/Accumulation.glsl:22-30). */
    AGB_ACCUM_RUNNING_MEAN = 1,
    /* FP32 Kahan-compensated sum and sample count; resolve divides. */
    AGB_ACCUM_KAHAN = 2,
    /* Per-pixel sum of sample luminance and of its square (FP32), for the denoiser's variance
     * feature. */
    AGB_ACCUM_MOMENTS = 4
};

/* Wave sizing (agb_render_options.max_paths_in_flight). */
#define AGB_WAVE_LARGEST 0xFFFFFFFFu
#define AGB_WAVE_DEFAULT_BYTES (8ull << 30)

/* Render options beyond FrameData. */
typedef struct agb_render_options
{
    uint32_t width;
    uint32_t height;
    uint32_t accumulation;      /* AGB_ACCUM_* bitmask */
    uint32_t max_paths_in_flight; /* wave size in paths; 0 = the call's samples in as few waves
                                     as fit in AGB_WAVE_DEFAULT_BYTES of wave buffers;
                                     AGB_WAVE_LARGEST = as few waves as fit in half the free
                                     device memory (at most a third of the device); either is
                                     halved again if allocation fails */
    int32_t env_filter_linear;  /* environment sampler: 0 nearest (Hgi default), 1 bilinear */
    uint32_t seed_offset;       /* added to the sample index that seeds the random streams, not to
                                   the accumulation index (gSampleData.seedOffset,
                                   MainEntryPoints.slang:83; PTRenderer.cpp:1008-1022) */
    int32_t _pad[2];
} agb_render_options;

typedef struct agb_context agb_context;

/* Per-render statistics, filled by agb_render when stats is non-null (the call then waits for the
 * render to finish). */
typedef struct agb_render_stats
{
    uint64_t paths;               /* camera paths traced */
    uint64_t closest_rays;        /* closest-hit rays traced (all segments) */
    uint64_t shadow_rays;         /* shadow rays traced */
    uint64_t node_visits;         /* closest-hit BVH node visits (when counting is enabled) */
    uint64_t tri_tests;           /* closest-hit triangle tests (when counting is enabled) */
    uint64_t shadow_node_visits;  /* shadow-ray BVH node visits (when counting is enabled) */
    uint64_t shadow_tri_tests;    /* shadow-ray triangle tests (when counting is enabled) */
    uint64_t kernel_launches;     /* CUDA kernels launched by this call */
    double gpu_ms;                /* device time of the call (CUDA events) */
    /* Device time per kernel family (when profiling is enabled): camera, closest-hit traversal,
     * shading, shadow traversal, resolve, finalize. */
    double kernel_ms[6];
    uint64_t kernel_count[6];     /* launches per kernel family */
    uint64_t shading_points;      /* hits shaded through the BSDF (the surface kernel's points) */
    uint64_t closest_rays_per_bounce[16]; /* closest-hit rays of bounces 0-15 (summed over waves) */
    uint64_t shadow_rays_per_bounce[16];  /* shadow rays of bounces 0-15 */
} agb_render_stats;

/* ------------------------------------------------------------------------------------------ */
/* Context.                                                                                    */
/* ------------------------------------------------------------------------------------------ */

/* Creates a renderer context on a CUDA device (replaces HGIRenderer construction,
 * HGI/HGIRenderer.cpp:36-62, and its Hgi device).  stream may be null (a stream is created). */
AGB_API agb_status agb_context_create(int32_t device, void* cuda_stream, agb_context** out);
AGB_API agb_status agb_context_destroy(agb_context* ctx);
/* Message of the last failing call on this thread (empty when none). */
AGB_API const char* agb_last_error(void);
/* Bytes of device memory the context holds. */
AGB_API agb_status agb_context_memory(agb_context* ctx, uint64_t* bytes);
/* Device bytes a render wave holds per path in flight (path state and ray / hit / shadow queues),
 * for hosts that size max_paths_in_flight or budget memory themselves.  No reference counterpart. */
AGB_API uint64_t agb_bytes_per_path(void);
/* A view renders the scene of ctx with its own stream (null: a new one), frame data and render
 * buffers (accumulation, AOVs, temporal history): several views of one resident scene render
 * concurrently.  Every render-side call (agb_frame_set, agb_render, agb_accum_read, ...) takes a
 * view in place of a context; scene calls on a view fail.  Views must be destroyed (with
 * agb_context_destroy) before their context.  No counterpart in the reference (its renderer owns
 * one render target set per scene); the serving loop uses it. */
AGB_API agb_status agb_view_create(agb_context* ctx, void* cuda_stream, agb_context** out);
/* Enables device-side counting of node visits / triangle tests (for the roofline). */
AGB_API agb_status agb_set_counting(agb_context* ctx, int32_t enabled);
/* Enables per-kernel-family device timing with CUDA events (agb_render_stats::kernel_ms). */
AGB_API agb_status agb_set_profiling(agb_context* ctx, int32_t enabled);

/* ------------------------------------------------------------------------------------------ */
/* Scene.                                                                                      */
/* ------------------------------------------------------------------------------------------ */

/* Copies one triangle mesh to the device and builds its BLAS (replaces HGIGeometry::update,
 * HGI/HGIGeometry.cpp:35-161).  Host pointers; normals/texcoords may be null; indices may be null
 * for non-indexed geometry (sequential indices, HGIGeometry.cpp:37-47).  index_count is 3 x
 * triangles (vertex_count when indices is null). */
AGB_API agb_status agb_geometry_create(agb_context* ctx, const float* positions,
    const float* normals, const float* texcoords, const uint32_t* indices, uint32_t vertex_count,
    uint32_t index_count, int32_t* out_geometry);

/* BVH builder used by agb_geometry_create (BLAS) and agb_instances_set (TLAS; replaces the
 * acceleration-structure builds the reference hands to the driver, HGI/HGIGeometry.cpp:127-160,
 * HGI/HGIScene.cpp:377-420): AGB_BVH_GPU (default) builds on the GPU (binned SAH, breadth-first,
 * one CTA per node); AGB_BVH_HOST builds on the host (binned SAH, depth first).  The TLAS has one
 * instance per leaf and takes the depth the deepest BLAS leaves on the traversal stack (splits
 * fall back to the index midpoint near that budget); a scene whose instance count needs more
 * levels than that is refused with AGB_ERR_LIMIT.  Both builders produce the same node layout
 * and depth bound; any valid BVH gives the same hits. */
enum
{
    AGB_BVH_HOST = 0,
    AGB_BVH_GPU  = 1
};
AGB_API agb_status agb_set_bvh_builder(agb_context* ctx, int32_t builder);
/* Reads a geometry's BLAS back (tests, tools): nodes (16 floats each: child 0 x lo / hi, y lo / hi;
 * child 1 the same; z lo / hi of both children; the two child refs as int bits, 2 unused), the
 * triangles in leaf order (12 floats each: v0 with the triangle id as int bits in w, v1, v2),
 * the root ref (a node index, or a leaf ref ~(first << 3 | count - 1)), depth and node count.
 * Either array may be null. */
AGB_API agb_status agb_geometry_bvh(agb_context* ctx, int32_t geometry, float* nodes_out,
    uint64_t node_capacity, float* tris_out, uint64_t tri_capacity, int32_t* root, int32_t* depth,
    uint32_t* node_count);

/* Reads the context's TLAS back (tests, tools): nodes as agb_geometry_bvh writes them, the
 * instance index of each leaf slot (a leaf ref ~(slot << 3) names slot), root ref, depth, node
 * count.  Either array may be null.  No reference counterpart (the driver owns its TLAS). */
AGB_API agb_status agb_tlas_read(agb_context* ctx, float* nodes_out, uint64_t node_capacity,
    int32_t* order_out, uint64_t order_capacity, int32_t* root, int32_t* depth, uint32_t* node_count);

/* Uploads an image (material texture or environment).  Host pixels, rows top to bottom.
 * linear: 1 bilinear, 0 nearest filtering (repeat addressing). */
AGB_API agb_status agb_image_create(agb_context* ctx, const void* pixels, uint32_t width,
    uint32_t height, int32_t format, int32_t linear, int32_t* out_image);

/* Replaces the material table (HGIMaterial::update uploads, HGI/HGIMaterial.cpp:23-60).
 * textures may be null. Host arrays of count entries. */
AGB_API agb_status agb_materials_set(agb_context* ctx, const agb_material* materials,
    const agb_material_textures* textures, uint32_t count);

/* Material node graphs.  The reference generates shader code from a MaterialX document's node
 * graphs (MaterialX/BSDFCodeGenerator.cpp:55-140 binds texcoord, normal, tangent and object /
 * world position to the generated code; MaterialGenerator.cpp:30-120 routes the graph outputs
 * into the material's fields).  Here the host compiles a graph into a program of register
 * operations over float4 registers (AGB_GRAPH_REGS of them) that the shading runs per hit, after
 * the material's constants and textures are read, writing the fields the graph drives.
 * Operations (r = registers, K = the constants, all component-wise unless stated):
 *   CONST    r[dst] = K[imm]
 *   INPUT    r[dst] = hit attribute imm (AGB_GIN_*; texcoord as (u, v, 0, 0), vectors with w = 0)
 *   ADD SUB MUL DIV MIN MAX  r[dst] = r[a] op r[b];  POW r[dst] = pow(r[a], r[b]);
 *   MOD      r[dst] = r[a] - r[b] * floor(r[a] / r[b])
 *   FLOOR CEIL ABS SIN COS SQRT SIGN  r[dst] = f(r[a])
 *   CLAMP    r[dst] = min(max(r[a], r[b]), r[c])
 *   MIX      r[dst] = r[b] + r[c] * (r[a] - r[b])        (fg = a, bg = b, mix = c)
 *   DOT      r[dst] = splat(sum over the first d components of r[a] * r[b], in order)
 *   NORMALIZE r[dst] = the first d components of r[a] / sqrt(dot), the rest 0
 *   LENGTH   r[dst] = splat(sqrt(dot of the first d components))
 *   SWIZZLE  r[dst] = (r[a][imm & 3], r[a][(imm >> 2) & 3], r[a][(imm >> 4) & 3], r[a][(imm >> 6) & 3])
 *   COMBINE  r[dst] = (r[a].x, r[b].x, r[c].x, r[d].x)
 *   SELECT   r[dst] = (r[a].x cmp r[b].x) ? r[c] : r[d], cmp = imm (0 >, 1 >=, 2 ==)
 *   IMAGE    r[dst] = image imm sampled at r[a].xy (its own filter, repeat addressing)
 *   NORMALMAP r[dst] = normalize(T n.x + B n.y + N n.z), n = 2 r[a] - 1 with n.xy scaled by r[b].x,
 *            N the shading normal, T its tangent, B = normalize(cross(N, T))
 *   NOISE    r[dst] = splat(noise imm at r[a]): 0 Perlin noise of r[a].xy, 1 of r[a].xyz, 2 cell noise
 *            of r[a].xy, 3 of r[a].xyz (MaterialX's noise functions, stdlib mx_noise.glsl: the lookup3
 *            final mix as the lattice hash, improved-noise gradients and fade, scaled 0.6616 / 0.9820;
 *            cell noise = hash of the cell / 0xffffffff)
 *   OUTPUT   material field imm (AGB_GOUT_*) = r[a] */
enum
{
    AGB_GOP_CONST = 0, AGB_GOP_INPUT, AGB_GOP_ADD, AGB_GOP_SUB, AGB_GOP_MUL, AGB_GOP_DIV, AGB_GOP_MIN,
    AGB_GOP_MAX, AGB_GOP_POW, AGB_GOP_MOD, AGB_GOP_FLOOR, AGB_GOP_CEIL, AGB_GOP_ABS, AGB_GOP_SIN,
    AGB_GOP_COS, AGB_GOP_SQRT, AGB_GOP_SIGN, AGB_GOP_CLAMP, AGB_GOP_MIX, AGB_GOP_DOT,
    AGB_GOP_NORMALIZE, AGB_GOP_LENGTH, AGB_GOP_SWIZZLE, AGB_GOP_COMBINE, AGB_GOP_SELECT,
    AGB_GOP_IMAGE, AGB_GOP_NORMALMAP, AGB_GOP_OUTPUT, AGB_GOP_NOISE, AGB_GOP_COUNT
};
enum
{
    AGB_GIN_TEXCOORD = 0, AGB_GIN_POSITION_WORLD, AGB_GIN_POSITION_OBJECT, AGB_GIN_NORMAL_WORLD,
    AGB_GIN_NORMAL_OBJECT, AGB_GIN_TANGENT_WORLD, AGB_GIN_BITANGENT_WORLD, AGB_GIN_COUNT
};
enum
{
    AGB_GOUT_BASE_COLOR = 0, AGB_GOUT_SPECULAR_ROUGHNESS, AGB_GOUT_COAT_ROUGHNESS,
    AGB_GOUT_EMISSION_COLOR, AGB_GOUT_OPACITY, AGB_GOUT_NORMAL, AGB_GOUT_COUNT
};
#define AGB_GRAPH_REGS 32
#define AGB_GRAPH_MAX_OPS 4096
typedef struct agb_graph_op
{
    uint8_t op, dst, a, b, c, d; /* d: also the component count of DOT / NORMALIZE / LENGTH */
    uint16_t imm;
} agb_graph_op;
/* Programs for the current material table: material m runs ops[first[m] .. first[m] + count[m])
 * (count 0: none).  Register indices below AGB_GRAPH_REGS, constant and image indices valid,
 * at most AGB_GRAPH_MAX_OPS per program; checked here.  Replaced by the next call; cleared by
 * agb_materials_set.  Host arrays; constants 4 floats each. */
AGB_API agb_status agb_material_graphs_set(agb_context* ctx, const int32_t* first, const int32_t* count,
    uint32_t material_count, const agb_graph_op* ops, uint32_t op_count, const float* constants,
    uint32_t constant_count);

/* Replaces the instance list and rebuilds the TLAS (HGIScene::rebuildInstanceList and
 * rebuildAccelerationStructure, HGI/HGIScene.cpp:192-449). Host array. */
AGB_API agb_status agb_instances_set(agb_context* ctx, const agb_instance* instances,
    uint32_t count);

/* Sets the environment (HGIEnvironment / HGIImage alias-map build, HGI/HGIImage.cpp:45-90;
 * EnvironmentBase.cpp:52-71).  light_image / background_image: image handles or -1.  With a light
 * image, builds the alias table on the GPU from FP64 prefix sums and fills
 * light_tex_luminance_integral. */
AGB_API agb_status agb_environment_set(agb_context* ctx, const agb_environment_data* env,
    int32_t light_image, int32_t background_image);
/* Sets the scene's ground plane (IScene::setGroundPlanePointer, PTScene.cpp:660-667); null
 * removes it (the renderer's default plane is disabled, PTRenderer.cpp:713-727). */
AGB_API agb_status agb_ground_plane_set(agb_context* ctx, const agb_ground_plane* plane);
/* Reads back the environment alias table (width*height entries), the luminance integral the
 * shading divides by, and the FP64 luminance integral (either pointer may be null). */
AGB_API agb_status agb_environment_alias(agb_context* ctx, agb_alias_entry* host_out,
    uint64_t capacity, double* shading_integral, double* fp64_integral);

/* Layout of the table agb_environment_set builds.  AGB_ENV_TABLE_REFERENCE (default) reproduces
 * the reference's AliasMap::build bit for bit (FP32 sequential integral and sweep; the sweep runs
 * on one warp).  The reference's environment MIS reuses one random pair for the table bucket and
 * for the BSDF lobe choice (ShadeFunctions.slang:146,220,237), so its converged image depends on
 * the bucket layout, and matching its images needs its layout.  AGB_ENV_TABLE_FP64 builds the
 * table from FP64 prefix sums (exact texel distribution, FP64 integral). */
enum
{
    AGB_ENV_TABLE_REFERENCE = 0,
    AGB_ENV_TABLE_FP64      = 1
};
AGB_API agb_status agb_set_environment_table(agb_context* ctx, int32_t layout);

/* Builds the environment alias table like agb_environment_set (same kernels, same table and
 * integrals) without allocating any memory.  No counterpart in the reference: it is for hosts
 * that cannot allocate when the light image changes (a host whose device memory is all handed
 * out by its own allocator or budget, or one that must not stall other streams on cudaMalloc /
 * cudaFree).
 *   rgba_device  width*height RGBA32F texels in device memory, rows from the top, 16-byte aligned
 *   table_device width*height entries of device memory, 16-byte aligned
 *   layout       AGB_ENV_TABLE_REFERENCE or AGB_ENV_TABLE_FP64
 *   shading_integral, fp64_integral: host outputs, either may be null
 *   stream       a cudaStream_t of the current device (null: legacy default stream)
 * Scratch is one fixed array in the library's device image (about 12.6 MB, reserved by the CUDA
 * driver when it loads this part of the library), so width*height is at most
 * AGB_ENV_NOALLOC_MAX_TEXELS; larger images are rejected with AGB_ERR_LIMIT.  Works on the
 * current device.  Each call looks up the scratch address in the current context (no
 * allocation), so a context reset (cudaDeviceReset) is followed correctly; the first call on a
 * device can make the driver load this part of the library: make it before any stream capture.
 * Returns after the stream has finished the build.  All calls on a device share the one scratch
 * array: calls that overlap in time (two host threads, or two streams) race and corrupt each
 * other's tables, so callers serialise them. */
#define AGB_ENV_NOALLOC_MAX_TEXELS 262144u /* e.g. 512 x 512, 724 x 362 or 1024 x 256 */
AGB_API agb_status agb_environment_alias_build_noalloc(const float* rgba_device, uint32_t width,
    uint32_t height, int32_t layout, agb_alias_entry* table_device, double* shading_integral,
    double* fp64_integral, void* stream);

/* ------------------------------------------------------------------------------------------ */
/* Rendering.                                                                                  */
/* ------------------------------------------------------------------------------------------ */

/* Sets the per-frame data (replaces the FrameData UBO blit, HGI/HGIRenderer.cpp:502-513). */
AGB_API agb_status agb_frame_set(agb_context* ctx, const agb_frame_data* frame);

/* Renders sample_count samples starting at sample_start into the context's accumulation buffers
 * (replaces the HGIRenderer::render sample loop, HGI/HGIRenderer.cpp:494-587: ray dispatch +
 * accumulation).  sample_start == 0 restarts accumulation.  Asynchronous on the context stream. */
AGB_API agb_status agb_render(agb_context* ctx, const agb_render_options* options,
    uint32_t sample_start, uint32_t sample_count, agb_render_stats* stats);

/* Waits for the context stream (IRenderer::waitForTask, Aurora.h:1199). */
/* AGB_OK when all work queued on the context (or view) has finished, AGB_ERR_NOT_READY while some
 * is still running; never blocks. */
AGB_API agb_status agb_wait_poll(agb_context* ctx);
AGB_API agb_status agb_wait(agb_context* ctx);

/* Copies the accumulated image to the host as RGBA32F (IRenderBuffer::data, HGIRenderBuffer.cpp).
 * mode: AGB_ACCUM_RUNNING_MEAN reads the running mean; AGB_ACCUM_KAHAN reads sum / count. */
AGB_API agb_status agb_accum_read(agb_context* ctx, int32_t mode, float* host_rgba,
    uint64_t capacity_floats);
/* The same for a rectangle of the image (x0, y0, width, height), rows top to bottom: progressive
 * callers that track part of a large frame read only that part (no reference counterpart). */
AGB_API agb_status agb_accum_read_rect(agb_context* ctx, int32_t mode, uint32_t x0, uint32_t y0,
    uint32_t width, uint32_t height, float* host_rgba, uint64_t capacity_floats);
/* Device pointer to the accumulation buffer of a mode (RGBA32F, width*height*4 floats). */
AGB_API agb_status agb_accum_device(agb_context* ctx, int32_t mode, float** device_rgba);
/* Per-sample output of the last rendered sample (RGBA32F device buffer), like gResult. */
AGB_API agb_status agb_last_sample_device(agb_context* ctx, float** device_rgba);

/* Denoising AOVs (HitShaderEntryPoints.slang:149-233 for hits, MainEntryPoints.slang:115-118 and
 * :380-406 for ray generation and misses), produced by agb_render when the frame has
 * is_denoising_aovs_enabled, for the primary paths of the call's last sample (the reference keeps
 * the data of the last sample).  width*height each, rows from the top:
 *   depth_view            view-space depth (negative in front of the camera; sky_view_z on a miss)
 *   normal_roughness      guide normal xyz (unencoded), max(specular roughness, 0.05); on a miss
 *                         the reversed ray direction and 1
 *   base_color_metalness  base colour xyz, metalness; on a miss (0, 0, 0, 0.1)
 *   motion                previous-minus-current pixel position xy, view depth change, 0
 * agb_aov_read copies any of them to host memory (null = skip); agb_aov_device returns the device
 * arrays (valid until the next agb_render). */
typedef struct agb_aov_buffers
{
    const float* depth_view;
    const float* normal_roughness;
    const float* base_color_metalness;
    const float* motion;
} agb_aov_buffers;
AGB_API agb_status agb_aov_read(agb_context* ctx, float* depth_view, float* normal_roughness,
    float* base_color_metalness, float* motion);
AGB_API agb_status agb_aov_device(agb_context* ctx, agb_aov_buffers* out);

/* Temporal resolve (DirectX/Shaders/TemporalResolve.hlsl:97-249; settings as
 * PTRenderer.cpp:2035-2046, defaults alpha 1/16 .. 0.6 reaching the maximum at 6 pixels per
 * frame).  Resolves the running-mean accumulation of the last render (one jittered sample per
 * frame, camera jitter from agb_temporal_jitter) against the previous resolve, using that render's
 * AOVs (motion vectors, view depth); the history is reset on request, on the first call and when
 * the image size changes.  agb_temporal_read copies the resolved RGBA image; agb_post_process with
 * AGB_POST_SOURCE_TEMPORAL post-processes it. */
typedef struct agb_temporal_settings
{
    uint32_t is_reset;
    float blend_alpha_min;
    float blend_alpha_max;
    float speed_reference;
} agb_temporal_settings;
AGB_API agb_status agb_temporal_resolve(agb_context* ctx, const agb_temporal_settings* settings);
AGB_API agb_status agb_temporal_read(agb_context* ctx, float* host_rgba, uint64_t capacity);
/* The temporal resolve kernel over device arrays (parity tests): accum / history / out RGBA32F,
 * motion 4 floats and depth_view 1 float per pixel, width*height each; stream may be null. */
AGB_API agb_status agb_temporal_resolve_batch(const float* accum, const float* history,
    const float* motion, const float* depth_view, uint32_t width, uint32_t height,
    const agb_temporal_settings* settings, float* out, void* cuda_stream);
/* Tensor-core GEMM (tcgen05, BF16 operands, FP32 accumulation): D[M x N] = A[M x K] x B[N x K]^T,
 * all row-major device arrays (A, B as BF16 bit patterns).  M a multiple of 128, N a multiple of
 * 16 in [16, 256], K a positive multiple of 64.  The building block of the denoiser's
 * convolutions, exported for its parity tests.  Synchronises the stream. */
AGB_API agb_status agb_tc_gemm_bf16(const uint16_t* a, const uint16_t* b, float* d, int32_t m,
    int32_t n, int32_t k, void* cuda_stream);
/* 3x3 convolution on the tensor cores (the denoiser's layer), NHWC BF16 over a batch:
 * out[b][y][x][:] = bias + sum over taps and input channels of in[b][y+dy][x+dx][:] * w, zero
 * padded, optional ReLU; the input is the channel concatenation of in0 (read through a nearest 2x
 * upsample from height/2 x width/2 when up0) and in1 (may be null, c1 = 0).  c0, c1 and cout are
 * multiples of 16 (c0 >= 16, cout <= 1024); width even (height too with up0); wpack is the output
 * of agb_pack_conv_weights; out (BF16) and out32 (FP32) may each be null; inputs 16-byte and
 * outputs 32-byte aligned.  Exported for the denoiser's parity tests. */
AGB_API agb_status agb_conv3x3_bf16(const uint16_t* in0, const uint16_t* in1, const uint16_t* wpack,
    const float* bias, uint16_t* out, float* out32, int32_t batch, int32_t height, int32_t width,
    int32_t c0, int32_t c1, int32_t cout, int32_t up0, int32_t relu, void* cuda_stream);
/* agb_conv3x3_bf16 with the encoder's 2x2 average pool fused into its epilogue: also writes
 * pool[b][y/2][x/2][:] = bf16(0.25 * (((o(2y,2x) + o(2y,2x+1)) + o(2y+1,2x)) + o(2y+1,2x+1))) over the
 * BF16 outputs o (height and width even).  Exported for the denoiser's parity tests. */
AGB_API agb_status agb_conv3x3_pool_bf16(const uint16_t* in0, const uint16_t* in1, const uint16_t* wpack,
    const float* bias, uint16_t* out, uint16_t* pool, int32_t batch, int32_t height, int32_t width,
    int32_t c0, int32_t c1, int32_t cout, int32_t up0, int32_t relu, void* cuda_stream);
/* Weight gradient of agb_conv3x3_bf16 (same input arguments, cout <= 256, width even): adds
 * dw[tap][cin][cout] += sum over pixels of in[p + d(tap)][cin] * dy[p][cout] into the FP32 array dw. */
AGB_API agb_status agb_conv3x3_wgrad_bf16(const uint16_t* in0, const uint16_t* in1, const uint16_t* dy,
    float* dw, int32_t batch, int32_t height, int32_t width, int32_t c0, int32_t c1, int32_t cout,
    int32_t up0, void* cuda_stream);
/* Packs FP32 weights w[tap][cin][cout] (tap = 3 * (dy + 1) + (dx + 1)) for agb_conv3x3_bf16;
 * flip != 0 packs the data-gradient convolution instead (input = dY with cout channels, output = dX
 * with cin channels).  out holds 9 * cin * cout BF16 values. */
AGB_API agb_status agb_pack_conv_weights(const float* w, int32_t cin, int32_t cout, int32_t flip,
    uint16_t* out, void* cuda_stream);
/* ------------------------------------------------------------------------------------------ */
/* Learned denoiser (no counterpart in the reference, whose denoiser is NVIDIA NRD): a 4-level     */
/* U-Net on the tensor cores, trained on the renderer's own low / high sample-count pairs.        */
/* ------------------------------------------------------------------------------------------ */
/* Layers (3x3 convolutions, ReLU except the last), in parameter order, with (input channels ->
 * output channels) at resolution 1 / 2^level:
 *   0 x(16)->32 L0   1 32->32 L0   [2x2 average pool]   2 32->64 L1   3 64->64 L1   [pool]
 *   4 64->128 L2     5 128->128 L2 [pool]                6 128->256 L3 7 256->256 L3
 *   8 up(7)(256) + skip(5)(128) -> 128 L2   9 128->128 L2
 *  10 up(9)(128) + skip(3)(64) -> 64 L1    11 64->64 L1
 *  12 up(11)(64) + skip(1)(32) -> 32 L0    13 32->32 L0
 *  14 32->16 L0 (no ReLU; channels 0-2 are added to the log1p noisy input: the prediction of
 *     log1p(radiance))
 * Parameters: for each layer, w[9][cin][cout] (tap = 3 * (dy + 1) + (dx + 1)) then b[cout], FP32.
 * Features (16 BF16 channels per pixel, NHWC): log1p(noisy RGB), base colour, octahedral normal,
 * view depth / sky depth, log1p(luminance variance), 6 zeros.  Height and width multiples of 8. */
typedef struct agb_denoiser agb_denoiser;
AGB_API agb_status agb_denoiser_create(int32_t device, void* cuda_stream, uint64_t seed,
    agb_denoiser** out);
AGB_API agb_status agb_denoiser_destroy(agb_denoiser* dn);
AGB_API agb_status agb_denoiser_param_count(uint64_t* count);
AGB_API agb_status agb_denoiser_params(agb_denoiser* dn, float* host_out, uint64_t count);
AGB_API agb_status agb_denoiser_set_params(agb_denoiser* dn, const float* host, uint64_t count);
/* Gradients of the last training step (same layout as the parameters). */
AGB_API agb_status agb_denoiser_grads(agb_denoiser* dn, float* host_out, uint64_t count);
/* Inference on device features [batch][height][width][16]; writes the denoised RGBA radiance
 * (device, batch*height*width float4). */
AGB_API agb_status agb_denoiser_forward(agb_denoiser* dn, const uint16_t* features, int32_t batch,
    int32_t height, int32_t width, float* out_rgba);
/* One training step on a batch: forward, L1 loss on log1p radiance against target_rgba (device,
 * float4 per pixel), backward; update != 0 then applies Adam (beta 0.9 / 0.999, eps 1e-8) with the
 * learning rate.  *loss receives the mean L1 loss. */
AGB_API agb_status agb_denoiser_train_step(agb_denoiser* dn, const uint16_t* features,
    const float* target_rgba, int32_t batch, int32_t height, int32_t width, float learning_rate,
    int32_t update, float* loss);
/* The 16 feature channels of the context's last render (running mean; the frame must have had
 * is_denoising_aovs_enabled; the variance channel needs AGB_ACCUM_MOMENTS, else 0) into device
 * memory (width*height*16 BF16). */
AGB_API agb_status agb_denoiser_features(agb_context* ctx, uint16_t* out_features);
/* ------------------------------------------------------------------------------------------ */
/* Serving loop (no counterpart in the reference, whose progressive driver renders one view at a  */
/* time: Foundation/API/Aurora/Foundation/Timer.h:97-140, HdAuroraRenderPass.cpp:194-208).         */
/* ------------------------------------------------------------------------------------------ */
/* A persistent scheduler thread admits render requests of registered scenes as slots and HBM
 * budget free up (continuous batching: requests arriving while others render are admitted at
 * once), renders each through a pooled view of its scene on its own stream so requests overlap on
 * the device, and records queueing, rendering and total latency.  Scenes are contexts uploaded by
 * the caller, admitted by their HBM footprint (agb_server_add_scene fails with AGB_ERR_OOM beyond
 * the budget); a request reserves its render memory before it starts, and one that cannot fit even
 * with nothing else running fails with AGB_ERR_OOM.  The result is the running mean (RGBA32F) of
 * the request's samples, or the denoised image when AGB_SERVE_DENOISE is set and a denoiser is
 * attached (width and height multiples of 8).  Scenes must not change while the server runs;
 * these calls return status codes only. */
typedef struct agb_server agb_server;
enum
{
    AGB_SERVE_DENOISE = 1
};
typedef struct agb_serve_request
{
    int32_t scene;
    uint32_t width;
    uint32_t height;
    uint32_t spp;
    uint32_t seed_offset;
    int32_t flags;
    uint32_t _pad[2];
    agb_frame_data frame;
} agb_serve_request;
typedef struct agb_serve_result
{
    uint64_t id;
    agb_status status;
    uint32_t width;
    uint32_t height;
    int32_t _pad;
    double queue_ms;   /* submit -> start */
    double render_ms;  /* start -> result on the host */
    double latency_ms; /* submit -> result on the host */
} agb_serve_result;
AGB_API agb_status agb_server_create(int32_t device, uint64_t hbm_budget_bytes, int32_t max_slots,
    agb_server** out);
AGB_API agb_status agb_server_destroy(agb_server* srv);
AGB_API agb_status agb_server_add_scene(agb_server* srv, int32_t scene_id, agb_context* ctx);
AGB_API agb_status agb_server_set_denoiser(agb_server* srv, agb_denoiser* dn);
AGB_API agb_status agb_server_submit(agb_server* srv, const agb_serve_request* req, uint64_t* id);
/* Waits (timeout_ms < 0: without limit) for a request; fills result and copies its RGBA32F image
 * to host_rgba (may be null).  AGB_ERR_TIMEOUT when it did not finish in time (wait again); a
 * finished request is forgotten after this call. */
AGB_API agb_status agb_server_wait(agb_server* srv, uint64_t id, int32_t timeout_ms,
    agb_serve_result* result, float* host_rgba, uint64_t capacity);
AGB_API agb_status agb_server_memory(agb_server* srv, uint64_t* scene_bytes, uint64_t* render_bytes);
/* Batched rendering (no counterpart in the reference): several views or contexts, of one or
 * several scenes and of any resolutions, rendered by one wavefront, each stage one kernel launch
 * over the paths of all of them.  Every path carries its request: its scene (the scenes' BVHs,
 * materials and images share one device namespace built by the batch, rebuilt when a scene
 * changes), frame data, resolution, sample range and accumulation targets.  A view's image is the
 * one agb_render gives it alone (same random streams per pixel and sample).  The serving loop uses
 * this to merge the requests it has admitted.
 *   agb_batch_create: stream may be null (one is created); max_paths_in_flight bounds a wave (the
 *     requests' samples are split over several waves beyond it, each request taking a share in
 *     proportion to what it still needs).
 *   agb_batch_render: views[i] renders sample_counts[i] samples from sample_starts[i] (null: 0)
 *     with options[i] (width, height, accumulation, seed_offset; max_paths_in_flight and
 *     env_filter_linear are ignored) and the frame data set on it.  Views must not repeat, must
 *     agree on is_force_opaque_shadows_enabled, and their scenes must have no ground plane.
 *     Asynchronous: the views' own streams wait for the batch, so agb_accum_read and the denoiser
 *     calls on a view see its result; agb_batch_poll reports completion.  With stats it waits and
 *     fills them (paths, rays, launches, device time). */
typedef struct agb_batch agb_batch;
AGB_API agb_status agb_batch_create(int32_t device, void* cuda_stream, uint64_t max_paths_in_flight,
    agb_batch** out);
AGB_API agb_status agb_batch_destroy(agb_batch* batch);
AGB_API agb_status agb_batch_render(agb_batch* batch, agb_context* const* views,
    const agb_render_options* options, const uint32_t* sample_starts, const uint32_t* sample_counts,
    uint32_t count, agb_render_stats* stats);
/* Builds the batch's shared namespace over these scenes (contexts, not views) ahead of the renders:
 * later calls whose scenes are all among them reuse it (rebuilt only when one of them changes).
 * Without it, each call builds the namespace over its own scenes when they differ from the last
 * call's.  Waits for the batch's previous work. */
AGB_API agb_status agb_batch_set_scenes(agb_batch* batch, agb_context* const* scenes, uint32_t count);
/* AGB_OK once the last agb_batch_render has finished on the device, AGB_ERR_NOT_READY before. */
AGB_API agb_status agb_batch_poll(agb_batch* batch);
/* Per-kernel-family device times in agb_batch_render's stats (like agb_set_profiling). */
AGB_API agb_status agb_batch_set_profiling(agb_batch* batch, int32_t enabled);

/* Halton (2, 3) camera jitter in pixels, centred on [-0.5, 0.5] (PTRenderer.cpp:81-95,159-174):
 * index = (phase_count ? frame_index % phase_count : frame_index) + 1. */
AGB_API void agb_temporal_jitter(uint32_t frame_index, uint32_t phase_count, float out[2]);
/* agb_post_process source: the last temporal resolve instead of the accumulation. */
enum
{
    AGB_POST_SOURCE_TEMPORAL = 4
};

/* relMSE of the accumulation (mode as agb_accum_read) against a reference RGBA32F image in
 * device memory: mean over pixels and RGB of (x - r)^2 / (r^2 + eps), computed on the GPU in FP64
 * (a convergence monitor for progressive rendering). */
AGB_API agb_status agb_accum_rel_mse(agb_context* ctx, int32_t mode, const float* reference_device,
    double eps, double* out);

/* Post-processing (HGI/Shaders/PostProcessing.glsl:37-64): brightness, optional ACES, optional
 * sRGB approximation, alpha 1.  Writes RGBA32F (out_rgba32f) and/or RGBA8 (out_rgba8) host
 * buffers. */
AGB_API agb_status agb_post_process(agb_context* ctx, int32_t mode, const float brightness[3],
    int32_t tone_map, int32_t gamma, float* out_rgba32f, uint8_t* out_rgba8);

/* ------------------------------------------------------------------------------------------ */
/* Unit kernels over device arrays (used by the parity tests; stream may be null = default).   */
/* ------------------------------------------------------------------------------------------ */

/* Standard Surface BSDF over n shading points (StandardSurfaceBSDF.slang:598-1372).
 * op 0 evaluateMaterial(V, L); 1 sampleMaterial(V, rnd) -> L, pdf, lobe;
 * 2 evaluateMaterialAndPDF(V, L, rnd) -> pdf, lobe.  frames: 12 floats per point (normal, tangent,
 * bitangent, unused).  Vectors 3 floats, rnd 2 floats.  All device pointers. */
AGB_API agb_status agb_bsdf_batch(int32_t op, const agb_material* materials,
    const int32_t* material_index, const float* frames, const float* V, const float* L,
    const float* rnd, int64_t n, float* out_value, float* out_dir, float* out_pdf,
    int32_t* out_lobe, void* cuda_stream);

/* Ray casts against the context's scene: rays 8 floats (origin, tmin, direction, tmax; a negative
 * tmin is taken as 0);
 * out_tuv 3 floats (t or -1, u, v); out_inst_prim 2 ints.  any_hit: occlusion query.  Device. */
AGB_API agb_status agb_intersect_batch(agb_context* ctx, const float* rays, int64_t n,
    int32_t any_hit, float* out_tuv, int32_t* out_inst_prim);

/* Environment sampling through the context's alias table (Environment.slang:137-186):
 * rnd 2 floats -> radiance 3, direction 3, pdf 1.  Device pointers. */
AGB_API agb_status agb_env_sample_batch(agb_context* ctx, const float* rnd, int64_t n,
    float* out_radiance, float* out_dir, float* out_pdf);

/* PCG2D stream (Random.slang:96-137) for one pixel sample, n pairs.  Device pointer. */
AGB_API agb_status agb_random_stream(uint32_t sample_index, uint32_t screen_width, uint32_t px,
    uint32_t py, int32_t n, float* out, void* cuda_stream);

/* Library version string. */
AGB_API const char* agb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* AGB_H */
