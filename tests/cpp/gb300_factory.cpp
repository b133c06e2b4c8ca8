// Test scaffolding: vlm::create_backend / get_available_backends with the
// "gb300" branch a maintainer adds to vlm/src/vlm_backend.cpp:15-38.  The
// reference's own vlm_backend.cpp is compiled unmodified with its factory
// renamed (-Dcreate_backend=ref_create_backend
// -Dget_available_backends=ref_get_available_backends), so its non-virtual
// Backend methods (displace_wing, wake_shed, the multibody loads) link from
// the reference's source while this file answers the factory calls.
#include <memory>
#include <string>
#include <vector>

#include "vlm_backend.hpp"
#include "vlm_backend_gb300.hpp"

namespace vlm {
std::unique_ptr<Backend> ref_create_backend(const std::string& backend_name);

std::unique_ptr<Backend> create_backend(const std::string& backend_name) {
    if (backend_name == "gb300") return std::make_unique<BackendGB300>();
    return ref_create_backend(backend_name);
}

std::vector<std::string> get_available_backends() { return {"gb300"}; }
}  // namespace vlm
