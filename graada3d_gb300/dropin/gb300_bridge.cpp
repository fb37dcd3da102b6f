// Side table of library contexts for the drop-in translation units.
#include "gb300_bridge.h"

#include <cstdlib>
#include <mutex>
#include <unordered_map>

namespace gb300 {

namespace {
std::mutex g_mutex;
std::unordered_map<const void *, grada_ctx *> g_contexts;
std::unordered_map<const grada_ctx *, std::vector<uint64_t>> g_digests;

struct Cleanup {
  ~Cleanup() {
    for (auto &kv : g_contexts) grada_ctx_destroy(kv.second);
  }
} g_cleanup;
}  // namespace

grada_ctx *context_for(const void *owner) {
  std::lock_guard<std::mutex> lock(g_mutex);
  auto it = g_contexts.find(owner);
  if (it != g_contexts.end()) return it->second;
  const char *env = std::getenv("GRADA_DEVICE");
  const int device = env ? std::atoi(env) : 0;
  grada_ctx *ctx = nullptr;
  if (grada_ctx_create(device, &ctx) != GRADA_OK)
    throw std::runtime_error("grada_ctx_create failed on device " + std::to_string(device));
  g_contexts[owner] = ctx;
  return ctx;
}

void release(const void *owner) {
  std::lock_guard<std::mutex> lock(g_mutex);
  auto it = g_contexts.find(owner);
  if (it == g_contexts.end()) return;
  g_digests.erase(it->second);
  grada_ctx_destroy(it->second);
  g_contexts.erase(it);
}

std::vector<uint64_t> &upload_digests(grada_ctx *ctx) {
  std::lock_guard<std::mutex> lock(g_mutex);
  return g_digests[ctx];
}

void check(grada_ctx *ctx, int status, const char *what) {
  if (status != GRADA_OK)
    throw std::runtime_error(std::string(what) + ": " + grada_last_error(ctx));
}

}  // namespace gb300
