// FNV-1a hashes (registry.cpp snippet_hash) of the reference's variation snippets; an entry of
// a caller's variations.yaml is evaluated by the device code only when its hash matches.
// An empty table accepts every entry whose name, parameters and flags match.
#include "internal.h"

namespace rfk {
const std::map<std::string, uint64_t>& builtin_snippet_hashes() {
    static const std::map<std::string, uint64_t> h = {};
    return h;
}
}  // namespace rfk
