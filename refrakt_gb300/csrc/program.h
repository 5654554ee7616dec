// Layout of a compiled genome ("program") as the kernels read it, shared by host and device.
//
// The reference stages a flat float buffer of genome parameters into shared memory and
// runs per-genome GLSL generated from variations.yaml (src/flame.cpp:33-103,
// src/variation_table.cpp:217-264).  Here a genome compiles to a small word array instead:
// a header, then one block per xform holding the affine, post, colour terms and a list of
// (variation id, weight, parameter offset) entries that the kernel interprets.  Words are
// uint32; float fields are stored bit-cast.  One copy exists per temporal sample.
#pragma once

#include "rtc_types.h"

namespace rfk {

constexpr int kProgMaxWords = 4096;  // 16 KB staged per CTA
constexpr int kMaxXforms = 255;      // xform ids are traced as bytes
constexpr int kMaxParams = 1024;     // the reference's fp[1024] (flame.glsl:27, flame.cpp:73)
constexpr int kGroup = 256;          // walkers that share one xform draw (flame.cpp:15 BLOCK_WIDTH)
constexpr uint32_t kProgMagic = 0x52464b31u;  // "RFK1"

// header words
enum : int {
    H_MAGIC = 0,
    H_NX = 1,        // regular xforms
    H_HASFINAL = 2,
    H_WORDS = 3,     // total words
    H_WOFF = 4,      // offset of the normalised selection weights (NX floats)
    H_FINAL = 5,     // offset of the final xform block (0 if none)
    H_XOFF = 6       // NX block offsets follow
};

// xform block words
enum : int {
    X_NPRE = 0,      // pre_xform entries (applied to v before the precalcs)
    X_NTERM = 1,     // accumulated entries
    X_MASK = 2,      // precalc mask (PC_*)
    X_HASPOST = 3,
    X_AFF = 4,       // c00 c01 c10 c11 c20 c21 (flam3 coefs order)
    X_POST = 10,     // p00 .. p21
    X_COLOR = 16,
    X_CS = 17,       // color_speed
    X_OMCS = 18,     // 1 - color_speed, FP32
    X_OPACITY = 19,
    X_DRAWS = 20,    // RNG draws of one evaluation (first-run colour excluded)
    X_ROTF = 21,     // rotation_frequency (animate.tpl.glsl)
    X_TERMS = 22     // entries: (id | flags, weight, parameter word offset from block start)
};
constexpr uint32_t kTermNoWeightMul = 0x100u;  // entry flag: result not scaled by the weight

// precalc mask bits (variations.yaml:1-9 `common`)
enum : uint32_t {
    PC_R = 1u, PC_RSQ = 2u, PC_A = 4u, PC_PHI = 8u,
    PC_SINA = 16u, PC_COSA = 32u, PC_SINR = 64u, PC_COSR = 128u
};

// keyed-permutation tags of the walker shuffle schedule
enum : uint64_t { TAG_GLOBAL = 1, TAG_LOCAL = 2, TAG_TABLE = 3 };

}  // namespace rfk
