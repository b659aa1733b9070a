/* crt.h -- C ABI of the GB300-native cuda-rt ray-tracing hot path.
 *
 * One shared library (libcrt.so) built for sm_103a.  Plain pointers and
 * sizes only.  Unless a comment says otherwise, every pointer argument may
 * be host memory (pageable or pinned) or device memory; the library checks
 * which (cudaPointerGetAttributes) and copies as needed.  Calls that take a
 * `stream` are ordered on it (NULL = legacy default stream); calls that read
 * results into host memory synchronise that stream before returning.
 *
 * Every entry point returns a crt_status and never exits the process
 * (the reference prints and calls exit(1): src/scene.cpp:71-81).
 * crt_last_error_string() describes the last failure on the calling thread.
 *
 * Semantics follow the reference (mbartling/cuda-rt) bit for bit; each
 * declaration names the reference interface it replaces.
 */
#ifndef CRT_H_
#define CRT_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum crt_status {
  CRT_OK = 0,
  CRT_INVALID_ARG = 1,
  CRT_OOM = 2,
  CRT_CUDA_ERROR = 3,
  CRT_STACK_OVERFLOW = 4, /* a traversal stack overflowed (impossible below CRT_MAX_TRIANGLES) */
  CRT_TIMEOUT = 5,        /* a bounded device-side wait gave up */
  CRT_NOT_BUILT = 6,      /* the scene has no BVH yet */
} crt_status;

/* Largest triangle count one scene accepts.  It keeps every radix-tree depth
 * below 62, so the reference's 64-entry traversal stack (kernels/bvh.cu:379)
 * can never overflow. */
#define CRT_MAX_TRIANGLES (1 << 28)
/* Largest vertex (and normal) count: three coordinates per vertex keep every
 * float offset within int32. */
#define CRT_MAX_VERTICES (1 << 29)
/* Largest samples-per-pixel count of a render; an image holds at most 2^30
 * pixels (width * height). */
#define CRT_MAX_SPP (1 << 24)

typedef struct crt_scene crt_scene;

/* Material, inc/material.h:8-24: the fields Material::shade and
 * Light::shadowAttenuation read.  Trans() is isZero(kt), as in the
 * reference (inc/material.h:31). */
typedef struct crt_material {
  double ka[3], kd[3], ks[3], kt[3], ke[3];
  double shininess;
} crt_material;

/* A triangle mesh in FP32, indexed.  Replaces Scene_h (inc/scene.h:29-56):
 * vertices/normals are tinyobj's attrib_t arrays, the index arrays are
 * TriangleIndices' vertex_index / normal_index (inc/tris.h:9-13).
 * normal_indices may be NULL (then vertex_indices index the normals too);
 * material_ids may be NULL (every triangle uses material 0). */
typedef struct crt_mesh_desc {
  const float* vertices;   /* num_vertices * 3; num_vertices <= CRT_MAX_VERTICES */
  int32_t num_vertices;
  const float* normals;    /* num_normals * 3; num_normals <= CRT_MAX_VERTICES */
  int32_t num_normals;
  const int32_t* vertex_indices; /* num_triangles * 3 */
  const int32_t* normal_indices; /* num_triangles * 3 or NULL */
  int32_t num_triangles;
  const crt_material* materials; /* num_materials */
  int32_t num_materials;
  const int32_t* material_ids;   /* num_triangles or NULL */
} crt_mesh_desc;

/* The Camera getters the pixel kernel reads (inc/camera.h:26-40):
 * setfov (vertical, degrees), setFocalPoint, setFstop (aperture = 1/fstop;
 * INFINITY gives a pinhole).  eye is Camera::getEye, read only by the
 * specular term.  As in the reference, the camera sits at the origin and
 * looks down -z (kernels/raytracer.cu:126-154). */
typedef struct crt_camera {
  double fov;
  double focal_point;
  double fstop;
  double eye[3];
} crt_camera;

/* Light_h, inc/Light.h:7-29 (positional light; orientation unused). */
typedef struct crt_light {
  double color[3];
  double position[3];
  double radius;
  double constant_term, linear_term, quadratic_term;
} crt_light;

typedef struct crt_render_params {
  int32_t width, height;
  int32_t spp;                 /* samples per pixel, 1..CRT_MAX_SPP (the reference fixes 20: raytracer.cu:138) */
  int32_t row_begin, row_end;  /* rows [begin, end) counted from the top; 0,0 = all */
  uint32_t seed;               /* 0: the reference's per-pixel mrand streams (parity mode); any other
                                  value XORs seed * 0x9E3779B1 into each pixel's hash input
                                  (initPNRG, kernels/mrand.cu:38-41): an independent render */
} crt_render_params;

/* Outputs of crt_render.  Pixel (px, py), py counted from the top, is stored
 * at idx = (height - py - 1) * width + px, the reference's bottom-up order
 * (kernels/raytracer.cu:106).  Any pointer may be NULL. */
typedef struct crt_render_out {
  uint8_t* rgb8;     /* idx*3: (unsigned char)(255 * clamp(mean colour)) */
  float* rgb_f32;    /* idx*3: mean colour before clamping */
  int32_t* hit_id;   /* idx*spp + k: closest-hit triangle of sample k, -1 miss */
  double* hit_t;     /* idx*spp + k: its t */
  int32_t* shadow;   /* idx*spp + k: 1 occluded, 0 lit, -1 primary miss */
  double* rays;      /* (idx*spp + k)*6: primary ray origin, direction */
  uint64_t* traversal_stats; /* [2]: four-wide nodes visited, leaf triangles tested (all
                                rays of the call); non-NULL selects an instrumented kernel */
  double* rgb_f64;   /* idx*3: mean colour before clamping, in double */
  double* depth;     /* idx: mean over samples of the hit t (a miss counts 0) */
  int32_t* shadow_id; /* idx*spp + k: the occluding triangle when shadow is 1, else -1 */
} crt_render_out;

/* ---- scene lifetime: Scene_d::operator=(const Scene_h&) (src/scene.cpp:82-160)
 * uploads the mesh and builds the BVH; ~Scene_d (src/scene.cpp:163-171) frees.
 * crt_scene_create does both steps and synchronises `stream`.  The mesh arrays
 * may be host or device memory; the scene keeps its own copies.  Index arrays
 * in device memory are range-checked on the device before the build. */
crt_status crt_scene_create(const crt_mesh_desc* mesh, void* stream, crt_scene** out);
/* The same with the caller's device arrays borrowed, not copied: every array
 * of `mesh` must be device memory and stay valid, unchanged except as below,
 * until crt_scene_destroy (NULL normal_indices: the vertex indices index the
 * normals; NULL material_ids: material 0, in an array the scene allocates).
 * Vertices may be rewritten in place between calls; then
 * crt_scene_set_vertices(scene, NULL, rebuild, stream) refits or rebuilds
 * from them (a non-NULL array is refused, as is crt_scene_set_materials). */
crt_status crt_scene_create_borrowed(const crt_mesh_desc* mesh, void* stream, crt_scene** out);
crt_status crt_scene_destroy(crt_scene* scene);

/* New vertex positions for the same triangles (num_vertices * 3 floats),
 * then either a full LBVH rebuild (rebuild != 0) or an atomic bottom-up
 * refit on the existing topology (RefitBounds, kernels/bvh.cu:209-258).
 * Asynchronous on `stream`. */
crt_status crt_scene_set_vertices(crt_scene* scene, const float* vertices, int rebuild, void* stream);

/* ---- BVH: BVH_d::setUp / computeMortonCodes / sortMortonCodes / buildTree
 * (src/bvh.cpp:3-32, kernels/bvh.cu:260-292).  Asynchronous. */
crt_status crt_bvh_build(crt_scene* scene, void* stream);
/* RefitBounds on the current topology after the vertices changed in place. */
crt_status crt_bvh_refit(crt_scene* scene, void* stream);

/* Copies the build products in the reference's layout (inc/bvh.cuh:18-28):
 * nodes 0..N-2 internal, N-1..2N-2 leaves.  Host or device pointers, any
 * may be NULL; synchronises `stream`.
 *   scene_box[6]           findMinMax's mMin, mMax (kernels/scene.cu:72-85)
 *   codes[N], ids[N]       mortonCodes / object_ids after the sort
 *   nodes3[(2N-1)*3]       HNode parent, left, right (root parent = -1)
 *   node_boxes[(2N-1)*6]   sortedBBoxs lo xyz, hi xyz */
crt_status crt_bvh_export(crt_scene* scene, float* scene_box, int32_t* codes, uint32_t* ids, int32_t* nodes3,
                          float* node_boxes, void* stream);

/* ---- traversal: BVH_d::intersect (closest hit, kernels/bvh.cu:382-414)
 * and BVH_d::intersectAny (first hit in left-first DFS order,
 * kernels/bvh.cu:416-449).  rays: n * 6 doubles (origin, direction).
 * ids[n]: triangle id or -1; t[n]; normals[n*3] (closest only; the
 * smooth normal of bvh.cu:357-364).  t and normals may be NULL. */
crt_status crt_trace_closest(crt_scene* scene, const double* rays, int64_t n, int32_t* ids, double* t,
                             double* normals, void* stream);
crt_status crt_trace_shadow(crt_scene* scene, const double* rays, int64_t n, int32_t* ids, double* t,
                            void* stream);

/* ---- render: RayTracer::run + pullRaytracedImage (kernels/raytracer.cu:55-166,
 * inc/raytracer.h:53-63): thin-lens primary rays on the mrand stream,
 * closest hit, Material::shade with one shadow ray per hit, mean over the
 * samples, clamp, quantise.  Device memory: the first thin-lens render on a
 * device (finite fstop) also builds that device's thin-lens tables, 2.0 GB
 * held until the process exits, when 8 GB are free and no stream capture is
 * under way (see crt_set_lens_tables; crt_set_lens_tables(0) beforehand
 * keeps them off).  The renders of one scene (crt_render,
 * crt_render_recursive, crt_adjoint_lambert) share the scene's tile
 * counters: issue them on one stream, or order them, never overlapping. */
crt_status crt_render(crt_scene* scene, const crt_camera* camera, const crt_light* light,
                      const crt_render_params* params, const crt_render_out* out, void* stream);

/* ---- recursive render: traceRay with the reflection and refraction block
 * of kernels/raytracer.cu:196-237 (commented out in the reference, whose
 * renders therefore stop at shade()).  Below each primary ray, while depth
 * > 0, a material with kr != 0 adds kr % (the colour of the mirrored ray)
 * and then one with kt != 0 adds kt % (the colour of the refracted ray,
 * Snell's law with eta = 1/ior entering and ior leaving; none on total
 * internal reflection), each traced with depth - 1.  Secondary rays start
 * at the hit point with no offset and use crt_render's closest hit and
 * shade(); every shade() takes its three light draws from the pixel's mrand
 * stream in depth-first order.  The block's Refl()/Trans() tests are
 * isZero(kr)/isZero(kt) (inc/material.h:27-31), which would trace only
 * rays that add nothing; the intent (non-zero coefficient) is followed.
 * depth = 0 gives crt_render's image.  optics: num_materials entries (host
 * or device), or NULL for kr = ks (as Scene_h::LoadObj sets it,
 * src/scene.cpp:29) and ior = 1 (tinyobjloader's default).  Writes rgb8,
 * rgb_f32, rgb_f64, the primary rays' hit_id, hit_t and rays, and
 * traversal_stats as [0] rays traced for closest hits (primary, reflected
 * and refracted), [1] shadow rays; the other outputs must be NULL. */
#define CRT_MAX_DEPTH 8
typedef struct crt_optics {
  double kr[3]; /* Material::kr, inc/material.h:16 */
  double ior;   /* Material::ior (MTL Ni) */
} crt_optics;
crt_status crt_render_recursive(crt_scene* scene, const crt_camera* camera, const crt_light* light,
                                const crt_render_params* params, int32_t depth, const crt_optics* optics,
                                const crt_render_out* out, void* stream);

/* Thin-lens sample tables (no counterpart in the reference).  Each
 * thin-lens sample needs cos/sin(2*pi*u1) and sqrt(u2) in double for two
 * mrand draws (raytracer.cu:141-142); a draw takes one of 83,886,081
 * values, so the library tabulates both functions at every value once per
 * device (2.0 GB of device memory, built in about 6 ms by the same double
 * expressions) and the kernels load them instead of computing them.  Images
 * are identical either way.  On by default; built at the first thin-lens
 * render or batch creation on a device with 8 GB to spare, outside stream
 * capture, and held until the process exits.  enable = 0 turns them off for
 * later calls (the memory stays allocated). */
crt_status crt_set_lens_tables(int32_t enable);

/* Replace the material table (same count as at creation), e.g. new
 * per-triangle albedos.  Asynchronous. */
crt_status crt_scene_set_materials(crt_scene* scene, const crt_material* materials, int32_t num_materials,
                                   void* stream);

/* ---- differentiation (no counterpart in the reference): the adjoint of
 * crt_render's mean colour (rgb_f64) and depth with respect to the vertex
 * positions, the light position and each material's kd, for Lambert shading
 * with distance attenuation.  Interior gradients only: which triangle each
 * sample hits and whether its shadow ray is blocked are held fixed (no
 * visibility edges); the specular term is treated as constant.  The samples
 * are recomputed per tile (same rays, hits and shadow tests as the forward),
 * nothing is stored between the two.  Inputs: grad_rgb[W*H*3] = d loss /
 * d rgb_f64, grad_depth[W*H] = d loss / d depth (may be NULL).  Outputs are
 * overwritten: grad_vertices[num_vertices*3], grad_light[3],
 * grad_kd[num_materials*3] (any may be NULL).  Host or device pointers. */
crt_status crt_adjoint_lambert(crt_scene* scene, const crt_camera* camera, const crt_light* light,
                               const crt_render_params* params, const double* grad_rgb, const double* grad_depth,
                               double* grad_vertices, double* grad_light, double* grad_kd, void* stream);

/* ---- stage-level entry points (device pointers only) ----
 * Morton codes of each triangle's centroid (computeMortonCodesKernel,
 * kernels/bvh.cu:37-61), normalised by scene_box (6 floats, device).  Every
 * vertex index is range-checked on the device against num_vertices
 * (CRT_INVALID_ARG; such a triangle's vertices are not read and its code is
 * 0).  Synchronises `stream`. */
crt_status crt_morton(const float* vertices, int32_t num_vertices, const int32_t* vertex_indices,
                      int32_t num_triangles, const float* scene_box, int32_t* codes, void* stream);
/* Karras hierarchy (FindSpan / FindSplit / BuildHierarchy, kernels/bvh.cu:
 * 100-207) of n sorted codes, with `ids` the sorted triangle ids: nodes3
 * receives the (2n-1) HNode triplets (parent, left, right) in the reference's
 * numbering (internal 0..n-2, root 0 with parent -1; leaf n-1+k holds ids[k]
 * as left and right), as crt_bvh_export writes them.  Device pointers. */
crt_status crt_hierarchy(const uint32_t* codes, const uint32_t* ids, int32_t n, int32_t* nodes3, void* stream);
/* RefitBounds (kernels/bvh.cu:209-258) on given triplets: node_boxes
 * [(2n-1)*6] receives every node's box (leaf n-1+k: the box of triangle
 * ids[k]; internal: the union of its children), as crt_bvh_export writes
 * sortedBBoxs.  Every id and index is range-checked on the device
 * (CRT_INVALID_ARG).  Device pointers; synchronises `stream`. */
crt_status crt_refit(const float* vertices, int32_t num_vertices, const int32_t* vertex_indices, int32_t n,
                     const uint32_t* ids, const int32_t* nodes3, float* node_boxes, void* stream);
/* Stable ascending LSD radix sort of (key, value) pairs on the low
 * `key_bits` bits of the keys (thrust::sort_by_key, kernels/bvh.cu:267-273).
 * vals_in may be NULL: values are then 0..n-1.  Device pointers of the
 * current device.  It does not sort in place: an input array that overlaps
 * an output array, or two overlapping outputs, are refused with
 * CRT_INVALID_ARG.  Scratch is allocated per call (cudaMallocAsync); the call
 * synchronises `stream` and reports a look-back timeout as CRT_TIMEOUT. */
crt_status crt_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                          int32_t n, int32_t key_bits, void* stream);

/* No counterpart in the reference.  The same stable radix sort as
 * crt_sort_pairs, for callers that must not allocate device memory where they
 * sort: cudaMalloc synchronises the whole device (a per-frame rebuild would
 * stall on it every frame), some host frameworks forbid a plugin from
 * allocating on its own, and a hot-path sort must not fail with
 * out-of-memory mid-frame.  Its scratch is a fixed device array of about
 * 16.8 MB inside libcrt.so, held on every GPU that loads the library until
 * the process exits; n may not exceed CRT_SORT_NOALLOC_MAX_PAIRS (larger n:
 * CRT_INVALID_ARG, nothing launched).  No cudaMalloc/cudaFree or other
 * allocating call is made.  The first call in each CUDA context (per device,
 * and again after cudaDeviceReset) looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; with lazy module loading
 * that lookup also loads the library's device code, which places the array,
 * so the first call can fail with an out-of-memory CRT_CUDA_ERROR: make it at
 * initialisation, and before any stream capture.  All calls share the array:
 * each clears what must start at zero, and calls whose work overlaps on the
 * GPU race.  As crt_sort_pairs: device pointers of the current device, no
 * overlap between an input and an output array or between the outputs
 * (CRT_INVALID_ARG); synchronises `stream`. */
#define CRT_SORT_NOALLOC_MAX_PAIRS (1 << 20)
crt_status crt_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                                  uint32_t* vals_out, int32_t n, int32_t key_bits, void* stream);

/* Synchronise `stream` and report device-side errors the scene's kernels
 * recorded (stack overflow, bounded-wait timeout, non-finite input). */
crt_status crt_scene_check(crt_scene* scene, void* stream);

/* ---- batched form: no counterpart in the reference, whose main loop
 * (src/main.cpp:300-330) builds and renders one mesh per process.  Many
 * meshes, each with its own camera, light and image size, are built and
 * rendered by a persistent cooperative kernel: its phases (segmented
 * bounds, Morton codes, sort, split search and refit -- the same as
 * crt_bvh_build, per mesh -- then a render whose warps claim (mesh, pixel
 * tile) work items) are separated by grid-wide barriers with bounded waits.
 * The render runs in the same launch or in a persistent launch of its own
 * (crt_batch_tuning.launches; the autotuner picks the faster).
 * crt_batch_run captures the launches once into a CUDA graph and replays
 * them.  Every mesh's image is what crt_render gives for that mesh alone. */
typedef struct crt_batch crt_batch;

typedef struct crt_batch_view {
  crt_camera camera;
  crt_light light;
  int32_t width, height, spp;
} crt_batch_view;

/* Launch shape of the batch: block_size in {128, 256} threads (as many
 * blocks as fit on the GPU at once);
 * lanes_per_pixel in {1, 2, 4, 8, 16, 32}: the most lanes (rays traced at
 * once) a pixel may take, capped by its samples per pixel, so a warp covers
 * 32 / lanes pixels; stack = traversal-stack entries kept in shared memory
 * per thread (0, 8, 16), the rest in local memory; launches = 1: every
 * build phase and the render in one persistent cooperative launch, 2: the
 * build phases in one persistent cooperative launch and the render in a
 * persistent launch of its own (both captured in the same graph). */
typedef struct crt_batch_tuning {
  int32_t block_size, lanes_per_pixel, stack;
  float render_ms; /* written by crt_batch_autotune: the chosen shape's render time */
  int32_t launches;
} crt_batch_tuning;

/* Host meshes and views (num_meshes <= 1024).  Copies everything to one
 * device allocation, including the concatenated rgb8 images (mesh m's image
 * follows mesh m-1's, each in crt_render_out's bottom-up order). */
crt_status crt_batch_create(const crt_mesh_desc* meshes, const crt_batch_view* views, int32_t num_meshes,
                            void* stream, crt_batch** out);
crt_status crt_batch_destroy(crt_batch* batch);
/* Build every mesh's BVH and render every view (one or two launches).
 * use_graph != 0 replays a CUDA graph of them (captured on the first such
 * call after create or a tuning change).  rgb8 (host or device, NULL to skip) receives
 * the concatenated images; a host rgb8 synchronises `stream`. */
crt_status crt_batch_run(crt_batch* batch, int32_t use_graph, uint8_t* rgb8, void* stream);
crt_status crt_batch_set_tuning(crt_batch* batch, const crt_batch_tuning* tuning);
/* Times the render phase under each supported tuning (one launch of that
 * phase each, after a build and a warm-up render; lanes options that change
 * no mesh's lanes per pixel are skipped) and keeps the fastest. */
crt_status crt_batch_autotune(crt_batch* batch, crt_batch_tuning* chosen, void* stream);
/* Mesh `mesh`'s build products in crt_bvh_export's layout (host or device
 * pointers; any may be NULL).  Synchronises `stream`. */
crt_status crt_batch_export(crt_batch* batch, int32_t mesh, float* scene_box, int32_t* codes, uint32_t* ids,
                            int32_t* nodes3, float* node_boxes, void* stream);
/* Synchronise `stream` and report device-side errors of the last run. */
crt_status crt_batch_check(crt_batch* batch, void* stream);

/* ---- scene input and image output of the drop-in CLI (host only).
 * crt_obj_load reads a Wavefront OBJ and its MTL the way Scene_h::LoadObj
 * does through tinyobjloader (src/scene.cpp:6-58): polygons
 * fan-triangulated, per-face material ids (absent or unknown: material 0),
 * Ka/Kd/Ks/Kt(Tf)/Ke/Ns with tinyobjloader's defaults.  Vertex and normal
 * coordinates are rounded to FP32 (crt_mesh_desc's precision).  The MTL is
 * looked up in mtl_dir (NULL: the OBJ's directory).  Every face corner must
 * carry a normal index (the reference reads normals[-1] otherwise).  The
 * file is parsed in chunks of whole lines on all host cores (environment
 * variable CRT_OBJ_CHUNK_BYTES, default 262144, sets the chunk size; the
 * result and the first error reported do not depend on it).
 * crt_obj_mesh points a mesh description at the loaded arrays (valid until
 * crt_obj_free). */
typedef struct crt_obj crt_obj;
crt_status crt_obj_load(const char* obj_path, const char* mtl_dir, crt_obj** out);
crt_status crt_obj_mesh(const crt_obj* obj, crt_mesh_desc* mesh);
/* crt_obj_optics fills one crt_optics per material (crt_mesh_desc's
 * num_materials) for crt_render_recursive: kr = Ks, as Scene_h::LoadObj sets
 * it (src/scene.cpp:29), and ior = Ni (default 1). */
crt_status crt_obj_optics(const crt_obj* obj, crt_optics* optics);
crt_status crt_obj_free(crt_obj* obj);
/* writeBMP (src/bitmap.cpp:99-154): 24-bit BMP of a host rgb8 image in
 * crt_render_out's bottom-up order (rows padded to 4 bytes with zeros). */
crt_status crt_write_bmp(const char* path, int32_t width, int32_t height, const uint8_t* rgb8);

const char* crt_last_error_string(void);
const char* crt_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CRT_H_ */
