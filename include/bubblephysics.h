/*
 * bubblephysics.h - C ABI of the GB300-native bubble step (grid broadphase, radius-bounded
 * contact forces K_c / gamma, adaptive-substep damped leapfrog, LBVH rigid broadphase).
 *
 * This is the drop-in boundary for the reference's solver seam
 *   NativeMetalFrameExecuting.executeFrame(input: NativeSolverInput, scenarioStep:) -> NativeSolverFrame
 *   (Sources/BubblePhysicsNativeMetal/NativeSolverInput.swift:257-260)
 * which BubbleWorld.advance(by:) reaches through CompleteStepper.completeStep and NativePublicWorld.step
 * (Sources/BubblePhysicsPublic/BubbleWorld.swift:270-283, Sources/BubblePhysicsNativeMetal/NativePublicWorld.swift:162-258).
 *
 * Conventions
 *  - Plain C: no torch or CUDA types. Every pointer argument is HOST memory owned by the caller and the library
 *    owns all device memory, except in the allocation-free step and the rigid solver calls, which take the
 *    caller's DEVICE pointers. Records are plain structs whose sizes are pinned by static asserts in the
 *    implementation.
 *  - Bubbles are passed sorted by id (signed 64-bit, strictly increasing), segments sorted by id, like
 *    NativePublicWorld.step sorts them (NativePublicWorld.swift:248-249). Indices in every output refer to that order.
 *  - Every function returns an int status (bp_status). A step that fails publishes nothing: the world keeps the
 *    state of the last successful step (Sources/BubblePhysicsRuntime/CompleteStep.swift:5-7).
 *  - Calls are thread-compatible: one in-flight step per world / batch. Every device wait is bounded.
 */
#ifndef BUBBLEPHYSICS_GB300_H
#define BUBBLEPHYSICS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BP_ABI_VERSION 1

/* Status codes. Mirrors NativeMetalSolverError / NativeMetalWorldError
 * (NativeMetalSolver.swift:5-6, NativeSolverInput.swift:266-272). */
typedef enum bp_status {
    BP_OK = 0,
    BP_E_INVALID = 1,           /* invalidSnapshot: bad input record, unsorted ids, non-finite input */
    BP_E_SUBSTEP_LIMIT = 2,     /* substepLimitExceeded: 1024 substeps used with step time left */
    BP_E_NONFINITE = 3,         /* nonFinite: a bubble or contact field became non-finite */
    BP_E_CONTACT_VIOLATION = 4, /* contactViolation: pair d <= 0, centre inside immovable body, edge side change */
    BP_E_INFLIGHT = 5,          /* frameInFlight: a second step was requested while one is running */
    BP_E_TIMEOUT = 6,           /* a bounded device wait ran out (reported, context stays usable) */
    BP_E_CUDA = 7,              /* commandFailed: a CUDA runtime call failed */
    BP_E_CAPACITY = 8,          /* capacityOverflow: a size beyond the library's limits */
    BP_E_UNAVAILABLE = 9,       /* unavailable: no CUDA device / extension not built for this GPU */
    BP_E_ALLOC = 10,            /* allocationFailed */
    BP_E_WORLD_FAILED = 11      /* the world failed in an earlier step and is stopped */
} bp_status;

/* Substep limiter term (NativeMetalSubstepTerm, NativeSolverInput.swift:275). */
typedef enum bp_term { BP_TERM_REMAINING = 0, BP_TERM_STIFFNESS = 1, BP_TERM_DISTANCE = 2, BP_TERM_MARGIN = 3 } bp_term;

/* Contact-assertion violation kinds (NativeForceKernels nativeViolation*). */
typedef enum bp_violation { BP_VIOLATION_NONE = 0, BP_VIOLATION_PAIR = 1, BP_VIOLATION_INSIDE_BODY = 2,
                            BP_VIOLATION_EDGE_SIDE = 3 } bp_violation;

/* ---- records ------------------------------------------------------------------------------------------------ */

/* Bubble flags: NativePublicProperties.flags (NativePublicWorld.swift:69) + contact.w force-driven marker. */
enum {
    BP_BUBBLE_ENABLED = 1u,      /* publicFlags.x: the region policy applies */
    BP_BUBBLE_STATIC = 2u,       /* publicFlags.y: motion role .static (infinite mass, never moves) */
    BP_BUBBLE_WRAP = 4u,         /* publicFlags.z: region exit policy .wrap (else .remove) */
    BP_BUBBLE_FORCE_DRIVEN = 8u  /* contact.w: dynamic / motor / player roles feel global force, fields, gamma */
};

/* One bubble (NativeSolverBubble + NativePublicProperties; NativeMetalBufferLayout.swift:4-25). 80 bytes. */
typedef struct bp_bubble {
    int64_t id;                  /* ObjectID bit pattern as signed Int (NativePublicWorld.swift:194) */
    float center[2];
    float previous_center[2];    /* out: centre at the start of the last step (position.zw) */
    float velocity[2];
    float mass;
    float inverse_mass;          /* 0 = static */
    float radius;                /* target radius */
    float rotation;
    float angular_velocity;
    float contact_stiffness;     /* K_c (> 0 for contact) */
    float damping;               /* gamma, 1/s */
    uint32_t flags;              /* BP_BUBBLE_* */
    uint32_t category;           /* collision filter category bits */
    uint32_t mask;               /* collision filter mask bits */
    uint32_t region_result;      /* out: 0 unchanged, 1 removed by the region, 2 wrapped (publicFlags.w) */
    int32_t layer;               /* drawing layer (setLayer, Int32): a hit test answers with the highest layer */
} bp_bubble;

/* Segment flags (NativeMetalSegment.flags, NativeMetalBufferLayout.swift:63-79). */
enum {
    BP_SEGMENT_POLYGON_EDGE = 1u,  /* flags.w bit 0: one-sided static polygon edge with regions */
    BP_SEGMENT_CONVEX_START = 2u,  /* flags.w bit 1 */
    BP_SEGMENT_CONVEX_END = 4u,    /* flags.w bit 2 (informational) */
    BP_SEGMENT_HAS_OWNER = 8u,     /* flags.y */
    BP_SEGMENT_ALLOWED_SIDE = 16u, /* flags.z: fixed contact normal side (allowed_side) */
    BP_SEGMENT_KINEMATIC = 32u     /* flags.x (informational; segments do not move inside a step) */
};

/* One static segment (NativeSolverSegment + NativeSolverPolygonEdge). 64 bytes. */
typedef struct bp_segment {
    int64_t id;
    int64_t owner_id;
    float a[2];
    float b[2];
    float previous_start[2];     /* polygon edge: start of the previous edge of the ring (region.xy) */
    float outward_sign;          /* polygon edge: outward normal = left normal * sign (region.z) */
    float allowed_side;          /* collision.x when BP_SEGMENT_ALLOWED_SIDE */
    uint32_t flags;              /* BP_SEGMENT_* */
    uint32_t category;
    uint32_t mask;
    int32_t layer;               /* drawing layer of the owner polygon (a hit test answers with the highest layer) */
} bp_segment;

enum { BP_BODY_POLYGON = 0u, BP_BODY_CIRCLE = 1u, BP_BODY_CAPSULE = 2u };
enum { BP_BODY_STATIC = 1u, BP_BODY_KINEMATIC = 2u };

/* One rigid body that bubbles see as an obstacle: a static circle or capsule, or any kinematic body
 * (NativeRigidBody, NativeRigidPolygonState.swift:25-40). Dynamic bodies are rejected with bubbles
 * (NativeCompleteStepper.swift:71-88). Pose is the centre of mass at the START of the step; a kinematic body
 * advances by its velocity over the step inside the library (nativeRigidPredict, NativePostSolveKernels:65-80).
 * Vertices are local to the centre of mass. 80 bytes. */
typedef struct bp_body {
    int64_t id;
    float position[2];
    float angle;
    float bounding_radius;       /* physical.z: radius of the circle around the whole body */
    float velocity[2];
    float angular_velocity;
    float core_radius;           /* shape.y: circle / capsule radius around the core, 0 for a polygon */
    float half_length;           /* shape.z: capsule half axis */
    uint32_t kind;               /* BP_BODY_POLYGON / CIRCLE / CAPSULE */
    uint32_t flags;              /* BP_BODY_STATIC / BP_BODY_KINEMATIC */
    uint32_t vertex_offset;      /* into bp_world_input.body_vertices (float2 pairs) */
    uint32_t vertex_count;       /* polygon ring, 1 for a circle, 2 for a capsule */
    uint32_t triangle_offset;    /* into bp_world_input.body_triangles (uint32 triples) */
    uint32_t triangle_count;
    uint32_t category;
    uint32_t mask;
    int32_t layer;               /* drawing layer (setLayer, Int32): a hit test answers with the highest layer */
} bp_body;

/* Force field (NativeForceField, NativeForceKernels:11-17). 64 bytes. */
typedef struct bp_force_field {
    float position[2];
    float rotation;
    float falloff;
    float direction[2];          /* directional strength (local frame) */
    float strength;              /* radial / vortex strength */
    float radius;                /* reach of a circle field */
    uint32_t kind;               /* 0 directional, 1 radial, 2 vortex */
    uint32_t vertex_offset;      /* polygon shape: into field_vertices */
    uint32_t vertex_count;       /* 0 = circle */
    uint32_t filter_offset;      /* into field_object_ids (sorted) */
    uint32_t filter_count;
    uint32_t has_filter;
    uint32_t reserved[2];
} bp_force_field;

/* Rubber band of a player-driven bubble (NativeBandDrive). Sorted by bubble_id. 24 bytes. */
typedef struct bp_band {
    int64_t bubble_id;
    float target[2];
    float stiffness;             /* K_band */
    float maximum_force;         /* 0 = unlimited */
} bp_band;

/* Motor of a motor-driven bubble (NativeMotor). Sorted by bubble_id. 24 bytes. */
typedef struct bp_motor {
    int64_t bubble_id;
    float force[2];
    float torque;
    float inertia;
} bp_motor;

/* World flags (package switches of NativeMetalConfiguration, NativeMetalSubstepLoop.swift:276-308). */
enum {
    BP_WORLD_HAS_REGION = 1u,          /* apply the public region exit policy at the end of the step */
    BP_WORLD_MINIMUM_MARGIN_ONLY = 2u, /* minimumMarginOnly: margin r/4 only (a rebuild almost every substep) */
    BP_WORLD_ASSERT_EVERY_SUBSTEP = 4u,/* assertEverySubstep */
    BP_WORLD_INJECT_STATE = 8u,        /* injectedSubstepState (diagnostic, host-chosen position) */
    BP_WORLD_NO_END_ASSERTION = 16u,   /* skip the end-of-step contact assertion (it is on by default) */
    BP_WORLD_FORCE_MULTI_CTA = 32u,    /* forceMultipleDispatches: step on the whole-GPU path even when small */
    BP_WORLD_RIGID_TREE = 64u,         /* find rigid candidates through the LBVH whatever the world's size */
    BP_WORLD_NO_RIGID_TREE = 128u      /* find rigid candidates by brute force whatever the world's size */
};

/* Per-world configuration (NativeSolverConfiguration + NativeMetalConfiguration). 64 bytes. */
typedef struct bp_world_desc {
    float time_step;                 /* dt of one step */
    float separation_tolerance;      /* sepTol, default 0.002 */
    float contact_tolerance;         /* default 0.001 */
    float substep_split_multiplier;  /* < 1 means 1 */
    float region[4];                 /* min.xy, max.xy (with BP_WORLD_HAS_REGION) */
    float global_force[2];           /* force on every force-driven bubble (then x inverse mass) */
    float gravity[2];                /* acceleration added to force-driven bubbles (0 = reference behaviour) */
    uint32_t candidate_limit;        /* k: candidates / neighbours per object, 1..128 (default 128) */
    uint32_t flags;                  /* BP_WORLD_* */
    int64_t inject_object;           /* BP_WORLD_INJECT_STATE: bubble id */
} bp_world_desc;

typedef struct bp_world_diagnostics {
    uint32_t inject_substep;         /* substep of the frame (from 0) after which the state is injected */
    float inject_position[2];
    uint32_t reserved;
} bp_world_diagnostics;

/* Everything a world needs besides its configuration. Arrays may be NULL when their count is 0. */
typedef struct bp_world_input {
    const bp_bubble* bubbles;        uint32_t bubble_count;
    const bp_segment* segments;      uint32_t segment_count;
    const bp_body* bodies;           uint32_t body_count;
    const float* body_vertices;      uint32_t body_vertex_count;    /* float2 pairs */
    const uint32_t* body_triangles;  uint32_t body_triangle_count;  /* uint32 triples */
    const bp_force_field* fields;    uint32_t field_count;
    const float* field_vertices;     uint32_t field_vertex_count;   /* float2 pairs */
    const int64_t* field_object_ids; uint32_t field_object_id_count;
    const bp_band* bands;            uint32_t band_count;
    const bp_motor* motors;          uint32_t motor_count;
    /* Joint exclusion lists (pairs joined without collideConnected have no contact; nativeJointExcluded).
     * One (start, count) pair per entity: bubbles first, then bodies; partners are object ids. */
    const uint32_t* joint_ranges;    uint32_t joint_entity_count;
    const int64_t* joint_partners;   uint32_t joint_partner_count;
} bp_world_input;

/* Result of one step (NativeMetalFrameTelemetry + failure detail, NativeMetalSubstepLoop.swift:346-396). 96 bytes. */
typedef struct bp_step_report {
    int32_t status;                  /* bp_status of this step */
    uint32_t substep_count;          /* substeps of this step (adaptive) */
    uint32_t rebuild_count;          /* grid rebuilds forced by the margin inside the step */
    uint32_t candidate_count;        /* candidates of the last grid build (pairs + segments) */
    uint32_t body_candidate_count;   /* bubble-body candidates of the last build */
    uint32_t candidate_overflow;     /* candidates dropped by the per-object limit k (max over builds) */
    uint32_t max_candidates_per_object;
    uint32_t contact_count;          /* active end-of-step contact records */
    uint32_t limiter_term;           /* bp_term of the last substep */
    uint32_t violation_kind;         /* bp_violation */
    int64_t limiter_object;          /* bubble id that set h in the last substep */
    int64_t violation_objects[2];
    int64_t violation_edge;          /* segment id (edge side violation) */
    float violation_distance;
    float cell_width;                /* grid cell width of the last build */
    float gpu_ms;                    /* device time of the step (batch: of the whole launch) */
    uint32_t removed_count;          /* bubbles removed by the region this step */
    uint32_t wrapped_count;
    uint32_t contact_overflow;       /* contact records beyond the world's record capacity (dropped) */
} bp_step_report;

/* End-of-step contact record (NativeContactCache, NativeGeometryKernels:26-29). 64 bytes. */
typedef struct bp_contact {
    int64_t participants[2];         /* bubble id, bubble id / segment id */
    uint32_t kind;                   /* 0 bubble-bubble, 1 bubble-segment */
    uint32_t feature;                /* polygon edge feature: 0 none, 1 interior, 2 convex start vertex */
    float normal[2];
    float point[2];
    float impulse;                   /* F * dt^2 (response.x) */
    float penetration;               /* response.y */
    float allowed_side;              /* response.z */
    uint32_t reserved[3];
} bp_contact;

/* Candidate key (NativeContactKey, NativeMetalBufferLayout.swift:83-103): kind 0 pair, 1 segment, 2 body. 24 bytes. */
typedef struct bp_candidate_key {
    uint32_t kind;
    uint32_t reserved;
    int64_t first;
    int64_t second;
} bp_candidate_key;

/* ---- context ------------------------------------------------------------------------------------------------ */

typedef struct bp_context bp_context;
typedef struct bp_world bp_world;
typedef struct bp_batch bp_batch;

/* Version of this ABI (BP_ABI_VERSION). */
int bp_abi_version(void);
/* Human-readable name of a status code (static string). */
const char* bp_status_string(int status);
/* Whether a CUDA device this library can run on is present (BP_OK) or not (BP_E_UNAVAILABLE). */
int bp_device_available(int device);

/* A context binds one CUDA device and one stream (NativeMetalSolver(device:), NativeMetalSolver.swift:355). */
int bp_context_create(int device, uint32_t flags, bp_context** out);
int bp_context_destroy(bp_context* context);

/* ---- single world (plain per-world launch path; NativeMetalSolver.executeFrame) ------------------------------- */

/* Creates a world with its state resident on the device. Replaces NativeMetalSolver persistent state
 * (NativeMetalSolver.swift:122-139) + the first executeSnapshot upload (NativeMetalSolver.swift:461-466). */
int bp_world_create(bp_context* context, const bp_world_desc* desc, const bp_world_input* input, bp_world** out);
int bp_world_destroy(bp_world* world);
/* Overwrites the bubble records (same count and ids as created; e.g. a host-side transaction). */
int bp_world_write_bubbles(bp_world* world, const bp_bubble* bubbles, uint32_t count);
int bp_world_set_diagnostics(bp_world* world, const bp_world_diagnostics* diagnostics);
/* Advances `steps` steps of time_step each (one executeFrame per step; NativeMetalSubstepLoop.run,
 * NativeMetalSubstepLoop.swift:216-273). reports may be NULL, else holds `steps` entries. Stops at the first
 * failed step and returns its status. */
int bp_world_step(bp_world* world, uint32_t steps, bp_step_report* reports);
/* Readback of the published state (NativeMetalSolver.swift:1061-1067). */
int bp_world_read_bubbles(bp_world* world, bp_bubble* out, uint32_t capacity, uint32_t* count);
/* End-of-step contact records of the last step (NativeMetalSolver.swift:1041-1060). */
int bp_world_read_contacts(bp_world* world, bp_contact* out, uint32_t capacity, uint32_t* count);
/* Test seams: candidate keys of the last grid build sorted by key (NativeMetalSolver.swift:292-296) and the grid
 * cell (int64 x, y) of every bubble in the last build (nativeBuildGrid, NativeGeometryKernels:179-189). */
int bp_world_read_candidates(bp_world* world, bp_candidate_key* out, uint32_t capacity, uint32_t* count);
int bp_world_read_cells(bp_world* world, int64_t* out_xy, uint32_t capacity, uint32_t* count);
/* h of every substep of the last step (stepHistory, NativeForceKernels:730). */
int bp_world_read_substeps(bp_world* world, float* out, uint32_t capacity, uint32_t* count);
/* Sorted LBVH keys of the last step: (Morton code << 32) | leaf, leaves numbered segments first, then bodies; the
 * Morton code interleaves 15-bit quantized centres of the leaf boxes (x in the even bits) over the box of all centres.
 * Replaces the brute-force loops of nativeEmitBodyCandidates (NativeGeometryKernels:350-415) and the segment rule of
 * nativeFinishBubbleRow (NativeGeometryKernels:279-290) with a tree; *count = 0 when the last step used none
 * (fewer leaves than the automatic threshold, BP_WORLD_NO_RIGID_TREE, or a non-finite leaf box). */
int bp_world_read_rigid_keys(bp_world* world, uint64_t* out, uint32_t capacity, uint32_t* count);

/* ---- batch of independent worlds (one fused launch per step for all worlds) ----------------------------------- */

enum {
    BP_BATCH_PER_WORLD_LAUNCH = 1u, /* step each world with its own launch, one after another (the plain path) */
    BP_BATCH_USE_GRAPH = 2u,        /* capture the per-step launches in a CUDA graph and replay it */
    BP_BATCH_AUTOTUNE = 4u,         /* choose the block width, group-queue threshold and group width by timing on first
                                       use */
    BP_BATCH_NO_STAGING = 8u        /* step every world from global memory (no shared-memory workspace) */
};

typedef struct bp_batch_config {
    uint32_t flags;                  /* BP_BATCH_* */
    uint32_t threads_per_world;      /* threads per block of the persistent launch, 0 = automatic (autotuner or 256) */
    uint32_t warp_world_max;         /* worlds of at most this many bubbles go to the group queue (a group of
                                        group_width threads per world); 0 = automatic (autotuner or 64);
                                        UINT32_MAX = no group queue */
    uint32_t group_width;            /* threads of one group-queue team: 32, 64, 128 or 256, at most the block
                                        width; 0 = automatic (autotuner or 32) */
} bp_batch_config;

int bp_batch_create(bp_context* context, uint32_t world_count, const bp_world_desc* descs,
                    const bp_world_input* inputs, const bp_batch_config* config, bp_batch** out);
int bp_batch_destroy(bp_batch* batch);
/* Advances every live world `steps` steps. reports may be NULL, else world_count entries (status of the first
 * failure, or the last step; substep_count and rebuild_count summed over the steps; gpu_ms = device time of the
 * whole call, measured with events on the library's stream). Worlds that fail stop; the others go on. */
int bp_batch_step(bp_batch* batch, uint32_t steps, bp_step_report* reports);
/* Total bubbles and total substeps x bubbles advanced since creation (for throughput). */
int bp_batch_counters(bp_batch* batch, uint64_t* bubble_count, uint64_t* bubble_substeps, uint64_t* launches);
int bp_batch_read_bubbles(bp_batch* batch, uint32_t world, bp_bubble* out, uint32_t capacity, uint32_t* count);
/* Bulk dynamic state of all worlds in world order: float4 (center.xy, velocity.xy) per bubble, in host memory.
 * write_state is queued on the library's stream and returns at once (the buffer must stay unchanged until the next
 * step or read completes); read_state returns when the data is in the buffer. A page-locked buffer (cudaHostAlloc or
 * cudaHostRegister), 16-byte aligned, is read or written by the kernels themselves across the host link; any other
 * buffer goes through a device staging array with a copy. */
int bp_batch_write_state(bp_batch* batch, const float* center_velocity, uint64_t bubble_count);
int bp_batch_read_state(bp_batch* batch, float* center_velocity, uint64_t bubble_count);
/* Sum of the adjacency degrees of all bubbles of the last grid build (mean degree = sum / bubbles); used to count
 * the algorithmic bytes of a substep. */
int bp_batch_adjacency_entries(bp_batch* batch, uint64_t* entries);
/* Schedule of the batched launch: [0] threads per block, [1] largest world of the group queue, [2] blocks of the
 * persistent launch, [3] worlds stepped by a whole block, [4] worlds of the group queue, [5] threads of one group. */
int bp_batch_tuning(bp_batch* batch, uint32_t* values, uint32_t count);

/* ---- contours (draw-only output of the step) ------------------------------------------------------------------ */

/* Contour parameters (NativeMetalContourControl.shape, NativeMetalBufferLayout.swift:175-178; defaults of
 * ReferenceConfiguration: maxContourSegmentLength 8, contourSurfaceTension 20, positionTolerance 1e-4). 16 bytes. */
typedef struct bp_contour_config {
    float max_edge;                  /* longest contour edge; samples per bubble = max(64, ceil(4 pi r / max_edge)) */
    float surface_tension;           /* smoothing weight tension / (tension + 10), at most 0.8 */
    float clearance;                 /* rays stop this far before a segment or chord */
    uint32_t stride;                 /* samples reserved per bubble; 0 = the largest sample count of the world */
} bp_contour_config;

/* ---- contact events (NativePublicWorld.contactTransitions, NativePublicWorld.swift:340-391) -------------------- */

/* A contact began / ended event. 48 bytes. objects: the pair, the smaller id (compared as unsigned 64-bit values)
 * first. For a began event: point = the records' penetration-weighted mean point, normal = their summed normal from
 * objects[0] towards objects[1], normalised, impulse = their summed F dt^2 divided by the step. */
typedef struct bp_contact_event {
    uint32_t kind;                   /* 0 began, 1 ended */
    uint32_t reserved;
    int64_t objects[2];
    float point[2];
    float normal[2];
    float impulse;
    float reserved2;
} bp_contact_event;

/* Contours of the world's published state, built on the device (nativeAccumulateContactPressure,
 * nativeGenerateContoursFused and nativePrepareRenderDataGrouped, NativePostSolveKernels:280-527: one ray per sample cut
 * by the one-sided segments and by the chord r (1 - eps) of every overlapping pair, 13 smoothing passes, the
 * bounded-slope majorant). Host outputs, each may be NULL: points_xy (bubble_count x stride float2), counts (samples
 * of each bubble; 0 for a removed one), level (bubble_count x stride deficits), shape (bubble_count x 6: largest
 * deficit, effective radius, bounds min.xy, max.xy). *stride_out = the stride used; with every output NULL the call
 * only reports it. gpu_ms (may be NULL) = device time of the kernel. Samples beyond a stride of 1024: BP_E_CAPACITY. */
int bp_world_contours(bp_world* world, const bp_contour_config* config, float* points_xy, uint32_t* counts,
                      float* level, float* shape, uint32_t* stride_out, float* gpu_ms);

/* Hit test of `count` query points (nativeHitTest, NativeGeometryKernels:501-541) on the published state: the bubbles
 * whose contour (built with `config`, as bp_world_contours) contains the point, the bodies that contain it and the
 * static polygons that contain it (the even-odd rule over each owner's polygon edges, which must be consecutive in
 * segment order, as bp_static_polygon_edges makes them) compete; the highest layer wins, then the largest id as an
 * unsigned 64-bit value. Per query: ids[q] (a bubble or body id, or a polygon's owner id), layers[q], found[q] (0 for
 * empty space). */
int bp_world_hit_test(bp_world* world, const bp_contour_config* config, const float* points_xy, uint32_t count,
                      int64_t* ids, int32_t* layers, uint32_t* found);

/* ---- sensors (enter / exit events of bubbles) ------------------------------------------------------------------ */

enum bp_sensor_flags {
    BP_SENSOR_ENTER_EVENTS = 1u,     /* report bubbles that start overlapping (sensor flag bit 2 of the reference) */
    BP_SENSOR_EXIT_EVENTS = 2u       /* report bubbles that stop overlapping (bit 3) */
};

/* A sensor (NativeSensorRecord, NativePostSolveKernels:586): a circle of `radius`, or a polygon of vertex_count local
 * vertices from bp_world_set_sensors' vertex array, at `position` rotated by `angle`. 48 bytes. */
typedef struct bp_sensor {
    int64_t id;
    float position[2];
    float angle;
    float radius;                    /* circle sensor (vertex_count 0) */
    uint32_t vertex_offset;          /* polygon sensor: into the vertex array (float2 pairs) */
    uint32_t vertex_count;
    uint32_t flags;                  /* BP_SENSOR_* */
    uint32_t reserved[3];
} bp_sensor;

/* One sensor event of the last step, in pair order (sensor, then bubbles, then bodies). 32 bytes. */
typedef struct bp_sensor_event {
    int64_t sensor;
    int64_t object;                  /* bubble or body id */
    uint32_t kind;                   /* 1 entered, 2 exited */
    float point[2];                  /* bubble centre or body position */
    uint32_t object_kind;            /* 0 bubble, 1 body */
} bp_sensor_event;

/* Sets the world's sensors (replacing any earlier ones). A pair is a sensor and one of the world's objects: its
 * bubbles in input order, then its bodies in input order; per-pair arrays hold one byte per pair, sensor-major.
 * allowed (may be NULL: every pair) is 1 where the sensor's object filter takes the object (the reference's
 * ObjectFilter.objectIDs, expanded per pair like NativeMetalSolver.swift:555-575); overlap_state (may be NULL: nothing
 * overlaps) is 1 where the pair overlapped before, so a host that rebuilds a world carries its sensors' state over.
 * Every later step compares each allowed pair on the device and lists the objects that entered or left: a bubble as in
 * nativeCompactSensorEvents (NativePostSolveKernels:601-648: within the summed radii of a circle sensor, inside a
 * polygon sensor or within its radius of an edge; removed bubbles overlap nothing), a body at its end-of-step pose as
 * in nativeCompactPolygonSensorEvents (:740-775: a circle or capsule core within its radius, a polygon's edges crossing
 * or touching, or either shape inside the other). */
int bp_world_set_sensors(bp_world* world, const bp_sensor* sensors, uint32_t count, const float* vertices_xy,
                         uint32_t vertex_count, const uint8_t* allowed, const uint8_t* overlap_state);
/* Sensor events of the last step; *count = all of them (capacity may be smaller). */
int bp_world_read_sensor_events(bp_world* world, bp_sensor_event* out, uint32_t capacity, uint32_t* count);

/* ---- serving loop (no counterpart in the reference) ------------------------------------------------------------ */

/* A request loop over many worlds that stay resident on the device. The reference steps one world per call
 * (NativePublicWorld.step -> executeFrame, NativeSolverInput.swift:257-260); a server takes step requests for any of
 * its worlds as they arrive and batches them continuously: every progress call finishes the batches whose device work
 * has ended, admits the worlds of waiting requests while the device memory budget allows (evicting the least recently
 * used idle worlds to pinned host memory, byte for byte, and bringing them back the same way), and launches one
 * persistent batched step over every ready world on one of its streams while earlier batches may still run. A world
 * has at most one step in flight; a request of n steps takes n batches. Results do not depend on the batching: a
 * world's state after its requests is the one bp_world_step gives. Worlds above 4096 bubbles are refused
 * (BP_E_CAPACITY). */
typedef struct bp_server bp_server;

enum bp_server_flags {
    BP_SERVER_PER_WORLD = 1u         /* one launch per world step, one at a time (the plain per-world path) */
};

/* 32 bytes. */
typedef struct bp_server_config {
    uint64_t hbm_budget_bytes;       /* device bytes of resident worlds; 0 = 120 GB */
    uint32_t max_worlds;             /* worlds the server can hold (resident or evicted) */
    uint32_t max_batch_worlds;       /* worlds per batched launch; 0 = no limit */
    uint32_t streams;                /* batches in flight at once; 0 = 8 */
    uint32_t threads_per_world;      /* block width for worlds stepped by a block (128, 256, 512); 0 = 512 */
    uint32_t warp_world_max;         /* worlds of at most this many bubbles go to the group queue (a group of
                                        group_width threads per world); 0 = 64, UINT32_MAX = none */
    uint32_t flags;                  /* BP_SERVER_* */
    uint32_t group_width;            /* threads of one group-queue team: 32, 64, 128 or 256; 0 = 32 */
    uint32_t reserved;
} bp_server_config;

/* A finished request. Times are seconds of bp_server_clock(). 136 bytes. */
typedef struct bp_server_completion {
    uint64_t request_id;
    uint32_t world;
    int32_t status;                  /* first failed step's status, else BP_OK */
    uint32_t steps;                  /* steps taken */
    uint32_t substeps;               /* substeps summed over the steps */
    double submitted_s, completed_s;
    bp_step_report report;           /* report of the last step taken */
} bp_server_completion;

/* Counters since creation. 80 bytes. */
typedef struct bp_server_stats {
    uint32_t worlds, resident;
    uint64_t resident_bytes, hbm_budget_bytes;
    uint64_t admissions, evictions, batches, batched_worlds, requests_done, bubble_substeps;
    double device_ms;                /* summed device time of the batches (events on their streams) */
} bp_server_stats;

int bp_server_create(bp_context* context, const bp_server_config* config, bp_server** out);
/* Waits for the work in flight, then frees every world. */
int bp_server_destroy(bp_server* server);
/* Registers a world (copied; it becomes resident when a request needs it). *world = its index. */
int bp_server_add_world(bp_server* server, const bp_world_desc* desc, const bp_world_input* input, uint32_t* world);
int bp_server_submit(bp_server* server, uint32_t world, uint32_t steps, uint64_t* request_id);
/* One round of the loop; waits up to wait_us for device work to finish when nothing else can be done.
 * *completed = requests finished in this round (may be NULL). */
int bp_server_progress(bp_server* server, uint32_t wait_us, uint32_t* completed);
/* Takes finished requests (oldest first); with out = NULL, *count = how many are waiting to be taken. */
int bp_server_poll(bp_server* server, bp_server_completion* out, uint32_t capacity, uint32_t* count);
/* Requests not yet finished: waiting for a batch, and worlds with a step in flight. */
int bp_server_pending(bp_server* server, uint32_t* waiting, uint32_t* in_flight);
/* State of one world (resident or evicted) after its finished steps. */
int bp_server_read_bubbles(bp_server* server, uint32_t world, bp_bubble* out, uint32_t capacity, uint32_t* count);
int bp_server_read_stats(bp_server* server, bp_server_stats* out);
/* Monotonic host clock in seconds (the time base of bp_server_completion). */
double bp_server_clock(void);

/* Contact began / ended events of the world's last step, compacted on the device from its contact records (bubble
 * pairs, and bubble-segment records reported as the segment's owner), then `extra` caller records (participants[0] a
 * bubble id, participants[1] the other object's id, normal from the bubble; e.g. bubble-body contacts the step does
 * not record). A record counts when its penetration or impulse is positive and either object is in interested_ids.
 * The world keeps the previous step's pair set (its contact history): began = pairs not in it, ended = its pairs that
 * are gone or lost an object in removed_ids (none when both were removed). Events are began (ascending pair), then
 * ended (ascending); the history becomes this step's pairs without removed objects. At most `capacity` events are
 * written, *count = all of them. step_seconds divides the impulses (the step's duration). */
int bp_world_contact_events(bp_world* world, const int64_t* interested_ids, uint32_t interested_count,
                            const int64_t* removed_ids, uint32_t removed_count, const bp_contact* extra,
                            uint32_t extra_count, float step_seconds, bp_contact_event* out, uint32_t capacity,
                            uint32_t* count);
/* Replaces the world's contact history (2 ids per pair, any order; e.g. when a world is rebuilt mid-run). */
int bp_world_set_contact_history(bp_world* world, const int64_t* pairs, uint32_t pair_count);
/* Reads the contact history (2 ids per pair, ascending pairs); with pairs = NULL, *count = the pair count. */
int bp_world_read_contact_history(bp_world* world, int64_t* pairs, uint32_t capacity, uint32_t* count);

/* ---- allocation-free step (no counterpart in the reference) ---------------------------------------------------- */

/* For callers that cannot allocate device memory while they step a world - a host framework that owns every device
 * allocation through its own pool, a real-time thread that must not take the driver's allocation locks, a process
 * that reserved all its device memory up front. The call allocates nothing: `bubbles` (bubble_count records, updated
 * in place to the published state after the steps), `segments` and `reports` (`steps` entries) are DEVICE pointers
 * owned by the caller, and every working array comes from one fixed 1 MiB device array built into the library (it
 * exists once on every GPU that loads the library, until the process exits).
 * Limits: at most 1024 bubbles, 256 segments, candidate limit at most 32 (0 means 32); no bodies, fields, bands,
 * motors or joints; injection and multi-CTA switches are ignored; rigid candidates always take the brute-force loops.
 * Larger inputs are rejected with BP_E_CAPACITY before anything runs.
 * Contact records: at most 4 per bubble + 64 are kept (contact_count stops there, the rest is counted in
 * contact_overflow, where bp_world_step keeps k per bubble + 64), and the records themselves are not returned.
 * Inputs: bubble ids must be strictly ascending (as bp_world_create requires); the kernel checks this and, if not,
 * steps nothing and writes BP_E_INVALID into every report. A bubble whose region_result is 1 (removed by the region
 * in an earlier call) stays removed, so consecutive calls continue one world; bp_world_create instead takes every
 * input bubble as live.
 * Runs on `stream` (a cudaStream_t, NULL = the default stream) on the current device and returns when the work is
 * queued; the step statuses are in `reports`. Every call looks up the array's device address with that device
 * current (a host-side lookup). Under lazy module loading, the first call in a process on a device loads the
 * library's device code, which allocates device memory for the code and the array: make that first call at setup
 * time, before any stream capture. Every call shares the one array and initialises what it needs, so calls must not
 * overlap on the GPU: two calls in flight at once race on it. */
int bp_world_step_noalloc(const bp_world_desc* desc, bp_bubble* bubbles, uint32_t bubble_count,
                          const bp_segment* segments, uint32_t segment_count, uint32_t steps,
                          bp_step_report* reports, void* stream);

/* ---- rigid body solver ------------------------------------------------------------------------------------------ */

/* The rigid solver's records, laid out like the reference's so its buffers bind unchanged. Bodies step once per step,
 * before the bubble substeps (NativeMetalSolver.swift:767-799): predict, body-pair candidates and CCD, then 8
 * iterations of {body contacts, apply, joints, apply joints, wall guard}; the finish runs after the bubble step.
 * Each entry below replaces one of those kernels (or kernel pairs) on the caller's device arrays. */

/* One rigid body (NativeRigidBody, NativeRigidPolygonState.swift:25-40 / NativeGeometryKernels:35-41). 160 bytes. */
typedef struct bp_rigid_body {
    uint64_t id;
    uint64_t reserved0;
    float pose[4];               /* centre of mass x, y, angle, angle at the start of the step */
    float previous[4];           /* centre of mass x, y at the start of the step; local centroid x, y */
    float motion[4];             /* velocity x, y, angular velocity, angular damping */
    float physical[4];           /* inverse mass, inverse moment of inertia, bounding radius, friction */
    uint32_t ranges[4];          /* vertex offset, vertex count, convex triangle offset, triangle count */
    uint32_t flags[4];           /* static, wraps at the region, region result (set here: 1 removed, 2 wrapped),
                                    restitution (float bits) */
    uint32_t filter[4];          /* category, mask, kinematic, layer */
    float shape[4];              /* core kind (0 polygon, 1 circle, 2 capsule), core radius, half length, reserved */
    float limits[4];             /* maximum linear speed, maximum angular speed (0 = none), CCD marker, reserved */
} bp_rigid_body;

/* One joint (NativeJointRecord, NativeJointState.swift:7-14). Ends are entities: bubbles 0..n-1, then bodies n..;
 * BP_JOINT_WORLD_END is a world point (always end 0). Kind 0 distance, 1 hinge, 2 weld; flags 1 angle limits,
 * 2 motor. 96 bytes. */
#define BP_JOINT_WORLD_END 0xFFFFFFFFu
typedef struct bp_rigid_joint {
    uint64_t id;
    uint64_t reserved0;
    uint32_t ends[4];            /* end 0, end 1, kind, flags */
    float anchors[4];            /* anchor of end 0, anchor of end 1 (body-local frame, or a world point) */
    float parameters[4];         /* length, compliance, damping, reference angle */
    float limits[4];             /* lower and upper angle, motor target angular velocity, maximum torque */
    float state[4];              /* accumulated lambda of the step: distance, motor; two reserved */
} bp_rigid_joint;

/* Per-joint correction of the two ends (NativeRigidCorrection): pose delta and velocity delta. 64 bytes. */
typedef struct bp_rigid_correction {
    float first[4];
    float second[4];
    float velocity_first[4];
    float velocity_second[4];
} bp_rigid_correction;

/* A body stopped by its sweep against a wall owned by a static body (NativeRigidWall). 48 bytes. */
typedef struct bp_rigid_wall {
    int64_t participants[2];     /* body id, owner id of the wall */
    float geometry[4];           /* normal x, y; contact point x, y */
    float extra[4];              /* normal momentum stopped by the sweep x dt; three reserved */
} bp_rigid_wall;

/* One body-pair candidate of a body's row (NativeCandidate, NativeGeometryKernels:30): participants are the two
 * bodies' ids; metadata = (kind 3, lower body index, higher body index, float bits of the row's summed normal lambda
 * of the step). Rows are `row_width` entries per body, sorted by (kind, participants). 32 bytes. */
typedef struct bp_rigid_candidate {
    int64_t participants[2];
    uint32_t metadata[4];
} bp_rigid_candidate;

/* Safety bits OR-ed into *safety (the reference's safety word 3). */
enum {
    BP_RIGID_SAFETY_NONFINITE = 1u,         /* a pose or motion became non-finite */
    BP_RIGID_SAFETY_ROTATION_BUDGET = 18u,  /* 2 | 16: a predict sweep needed more than 128 rotation samples */
    BP_RIGID_SAFETY_INVALID = 256u          /* a record points outside its arrays: that body or joint is skipped
                                               (no counterpart in the reference, which reads past its buffers) */
};

/* Every pointer below is a DEVICE pointer owned by the caller; `stream` is a cudaStream_t (NULL = default stream).
 * The calls queue their work and return; they allocate nothing. `joint_ranges` holds one uint32 quadruple per entity
 * (bubbles first, then bodies): start and count in `references`, start and count in `joint_partners`;
 * `references` holds (joint index, side 0 or 1) pairs; `joint_partners` the sorted ids an entity does not collide
 * with. joint_ranges may be NULL (no joints); otherwise it holds bubble_count + body_count quadruples. Record arrays and
 * joint_ranges must be 16-byte aligned, vertices, references and partners 8-byte aligned (BP_E_INVALID otherwise). Rotations use the library's own float sin / cos
 * (Cody-Waite reduction by pi/2, Taylor series on |r| <= pi/4; absolute error below 1e-7 for |angle| <= 1000);
 * exponentials the float of the double-precision exp of the float argument. */

/* nativeRigidPredict (NativePostSolveKernels:66-115): start-of-step pose, damping and speed limits, integration; a
 * dynamic body sweeps its vertices against the segments (rotation sampled every 0.05 rad, at most 128 samples) and
 * stops, after a 12-step bisection, at the last pose without a crossing; a stop at a wall of a static body writes
 * walls[body]. bubble_count offsets the body entities in joint_ranges. Segments are static within the step. */
int bp_rigid_predict(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                     const bp_segment* segments, uint32_t segment_count, uint32_t bubble_count, float time_step,
                     const uint32_t* joint_ranges, const uint64_t* joint_partners, uint32_t partner_count,
                     bp_rigid_wall* walls, uint32_t* safety, void* stream);

/* `iterations` rounds of nativeSolveJoints then nativeApplyJointBodies (NativeContactKernels:446-562): every joint
 * computes both ends' corrections from the same state (XPBD distance with compliance and damping, hinge with limits
 * and motor, weld), then every body adds its joints' corrections in list order times 1 / count. A world of at most
 * 512 joints and 1,024 bodies runs all rounds in one launch, a larger one two launches per round; the results are
 * the same. iteration_count is the solver's iteration count per step (the damping is spread over it); a caller that
 * interleaves other work calls this with iterations = 1 each time. */
int bp_rigid_solve_joints(bp_rigid_body* bodies, uint32_t body_count, bp_rigid_joint* joints, uint32_t joint_count,
                          bp_rigid_correction* corrections, const uint32_t* references, uint32_t reference_count,
                          const uint32_t* joint_ranges, uint32_t bubble_count, float time_step,
                          uint32_t iteration_count, uint32_t iterations, uint32_t* safety, void* stream);

/* nativeRigidFinish (NativePostSolveKernels:172-198): non-finite check, speed limits, then the region policy from
 * the body's bounds (vertices plus core radius): removed (flags[2] = 1) or wrapped by whole region spans
 * (flags[2] = 2). region = (min x, min y, max x, max y), read on the host at the call. */
int bp_rigid_finish(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                    const float* region, uint32_t* safety, void* stream);

/* Body-pair rows (nativeRigidEmitCandidates in its body-pair mode, NativeGeometryKernels:394-415): for each body, the
 * other bodies (not both immovable, filters accepting, not joined without collideConnected) whose swept centre
 * distance comes within 1.25 x the sum of bounding radii; the `row_width` smallest keys are kept in order.
 * row_counts gets (entries, 0) per body; overflow[0] += dropped entries, overflow[1] = max(overflow[1], wanted). */
int bp_rigid_body_candidates(const bp_rigid_body* bodies, uint32_t body_count, uint32_t bubble_count,
                             const uint32_t* joint_ranges, const uint64_t* joint_partners, uint32_t partner_count,
                             uint32_t row_width, bp_rigid_candidate* rows, uint32_t* row_counts, uint32_t* overflow,
                             void* stream);

/* Body-body CCD (nativeRigidResolveCCD then nativeRigidApplyCCD, NativePostSolveKernels:200-263): every movable
 * body finds the earliest time of impact on its row's pairs (sampled every 0.5 units of travel, at most 64 samples,
 * 12 bisections; a pair overlapping at the start is left to the contacts), then moves back along its step to it.
 * `triangles` are uint32 quadruples (three indices into the body's vertex range, one unused), like the reference's
 * uint4 buffer; triangle_count counts quadruples. */
int bp_rigid_ccd(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                 const uint32_t* triangles, uint32_t triangle_count, const bp_rigid_candidate* rows,
                 const uint32_t* row_counts, uint32_t row_width, uint32_t* safety, void* stream);

/* One contact round (nativeRigidContacts then nativeRigidApplyBodies, NativeContactKernels:375-444): every row slot
 * computes its pair's contact (polygon triangles by SAT, circle / capsule cores, round against polygon) and the
 * pair's half position and velocity corrections with friction (geometric mean) and restitution (maximum), adding
 * the normal lambda to the slot's metadata[3]; then every body adds its row's corrections in order. `corrections`
 * has row_width entries per body. */
int bp_rigid_solve_contacts(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy,
                            uint32_t vertex_count, const uint32_t* triangles, uint32_t triangle_count,
                            bp_rigid_candidate* rows, const uint32_t* row_counts, uint32_t row_width,
                            bp_rigid_correction* corrections, uint32_t* safety, void* stream);

/* The wall guard (nativeRigidGuardWalls, NativePostSolveKernels:118-170): each dynamic body's vertices against the
 * static polygon bodies; a vertex that entered one (or crossed an edge within the step) is pushed out along the
 * nearest edge's normal and the approaching velocity is removed. */
int bp_rigid_guard_walls(bp_rigid_body* bodies, uint32_t body_count, const float* vertices_xy, uint32_t vertex_count,
                         const uint32_t* triangles, uint32_t triangle_count, uint32_t bubble_count,
                         const uint32_t* joint_ranges, const uint64_t* joint_partners, uint32_t partner_count,
                         uint32_t* safety, void* stream);

/* ---- host helpers (reference host logic that feeds the path) -------------------------------------------------- */

/* One-sided edges of a static polygon (NativeStaticPolygonEdges.segments, NativeStaticPolygonEdges.swift:16-37):
 * signed area in double, collinear merge at tolerance 1e-5, convex start/end, previous start. Writes at most
 * `capacity` segments with ids first_id, first_id+1, ... and returns the count in *count. */
int bp_static_polygon_edges(const float* points_xy, uint32_t point_count, int64_t first_id, int64_t owner_id,
                            uint32_t has_owner, bp_segment* out, uint32_t capacity, uint32_t* count);

/* Contact law on the device for known-answer tests (NativeMetalContactLawTests.swift:74-218).
 * mode 0: epsilon(q) of in[i].x; mode 1: wall law (K, r, d) -> (F, eps, k, 0);
 * mode 2: pair law (K_a, r_a, K_b, r_b, d) -> (F, eps_a, eps_b, k). in/out hold 8 floats per case. */
int bp_device_contact_law(bp_context* context, uint32_t mode, const float* in, float* out, uint32_t count);

#ifdef __cplusplus
}
#endif
#endif /* BUBBLEPHYSICS_GB300_H */
