// params.cpp - YAML parameters for the CPU oracle (TEST INFRASTRUCTURE ONLY).
//
// The oracle takes its parameters as a resolved xmd_params.  This links the
// engine's host-side parser (xmd_gb300/csrc/config.cpp, defaults_yml.cpp:
// plain C++, no CUDA) into liboracle.so, so that a CPU-only process, such as
// the benchmark's CPU arm, resolves a YAML file without mapping the engine
// library.  Same keys, units and merge over the defaults as
// xmd_gpu_parse_params.
#include <cstring>
#include <stdexcept>
#include <string>

#include "../xmd_gb300/csrc/config.h"

static thread_local std::string g_err;

extern "C" int xo_parse_params(const char *yaml_text, xmd_params *out) {
    if (!out) return XMD_ERR_ARG;
    try {
        xmdg::params_from_yaml(yaml_text ? yaml_text : "", out);
        g_err.clear();
        return XMD_OK;
    } catch (const std::exception &e) {
        g_err = e.what();
        return XMD_ERR_CONFIG;
    }
}

extern "C" const char *xo_last_error(void) { return g_err.c_str(); }
