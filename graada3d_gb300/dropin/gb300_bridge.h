// Bridge between the reference's C++ classes and the GB300 library.
//
// The reference's class headers (Fwd.h, GaussNewtonInversion.h) stay
// unchanged, so a library context cannot be a member: it lives in a side table
// keyed by the object's address.  One context per Fwd-derived object, created
// on first use on device 0 (GRADA_DEVICE overrides), released by
// gb300_release(owner) or at process exit.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/grada_gpu.h"

namespace gb300 {

grada_ctx *context_for(const void *owner);
void release(const void *owner);

// Throws std::runtime_error with the library's message on a failing status.
void check(grada_ctx *ctx, int status, const char *what);

// Digests of the inputs last uploaded to a context (the solve_cg drop-in skips
// unchanged uploads); dropped with the context by release().
std::vector<uint64_t> &upload_digests(grada_ctx *ctx);

// grada_build_operators' face table of a mesh (FaceTable_gb300.cpp).
}  // namespace gb300
class Mesh;
namespace gb300 {
void face_table(Mesh &mesh, std::vector<int32_t> &table);

}  // namespace gb300
