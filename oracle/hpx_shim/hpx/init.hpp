// Stand-in for hpx::init / hpx::local::finalize (reference lulesh.cc:2413-2437).
// Parses argv against the registered options, fills in defaults, and calls
// the program's hpx_main on the calling thread. Test infrastructure only.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include <hpx/hpx.hpp>
#include <hpx/modules/program_options.hpp>

int hpx_main(hpx::program_options::variables_map& vm);

namespace hpx {

struct init_params {
    program_options::options_description desc_cmdline;
};

namespace local {
inline int finalize() { return 0; }
}  // namespace local

inline int init(int argc, char** argv, const init_params& params) {
    namespace po = program_options;
    po::variables_map vm;
    const auto& desc = params.desc_cmdline;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a.rfind("--hpx:threads", 0) == 0) {
            std::string v;
            auto eq = a.find('=');
            if (eq != std::string::npos) v = a.substr(eq + 1);
            else if (i + 1 < argc) v = argv[++i];
            // The stand-in runs every task on one thread; the count is only
            // echoed back through get_num_worker_threads().
            detail::worker_threads() = v.empty() ? 1 : std::atoi(v.c_str());
            continue;
        }
        if (a.rfind("--hpx:", 0) == 0) continue;
        if (a.rfind("--", 0) != 0) {
            std::fprintf(stderr, "unexpected argument: %s\n", a.c_str());
            return 1;
        }
        std::string name = a.substr(2), val;
        bool have_val = false;
        auto eq = name.find('=');
        if (eq != std::string::npos) {
            val = name.substr(eq + 1);
            name = name.substr(0, eq);
            have_val = true;
        }
        const auto* opt = desc.find(name);
        if (!opt) {
            std::fprintf(stderr, "unknown option: --%s\n", name.c_str());
            return 1;
        }
        if (!opt->sem) {
            vm.set(name, std::any(true));
            continue;
        }
        if (!have_val) {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "option --%s needs a value\n", name.c_str());
                return 1;
            }
            val = argv[++i];
        }
        vm.set(name, opt->sem->parse(val));
    }
    for (const auto& o : desc.all())
        if (o.sem && o.sem->has_default() && !vm.count(o.name)) vm.set(o.name, o.sem->default_any());
    return hpx_main(vm);
}

}  // namespace hpx
