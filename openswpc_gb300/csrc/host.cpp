// host.cpp -- host driver layer (input files -> prepared simulation).
#include "../../include/swpc_gpu.h"
#include <string>
namespace swpc { int set_err(int code, const std::string& msg); }
extern "C" int swpc_host_prepare(const char* inf_path, swpc_sim** out) {
    (void)inf_path; if (out) *out = nullptr;
    return swpc::set_err(SWPC_E_STATE, "host driver layer not built yet");
}
extern "C" int swpc_host_write_sac(swpc_sim* sim, const char* odir) {
    (void)sim; (void)odir;
    return swpc::set_err(SWPC_E_STATE, "host driver layer not built yet");
}
extern "C" int swpc_host_nt(swpc_sim* sim) { (void)sim; return 0; }
