// Shared helpers of the command-line drivers: option parsing and status checks.
// The drivers call only the C ABI of include/bubbledyn.h.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

#include "bubbledyn.h"

namespace cli {

// --key value and --flag options; anything else is an error.
struct Args {
    std::map<std::string, std::string> kv;
    Args(int argc, char** argv, const char* usage) {
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i];
            if (a == "-h" || a == "--help") {
                std::printf("%s", usage);
                std::exit(0);
            }
            if (a.size() < 3 || a.compare(0, 2, "--") != 0) {
                std::fprintf(stderr, "unexpected argument %s\n%s", argv[i], usage);
                std::exit(2);
            }
            const std::string key = a.substr(2);
            if (i + 1 < argc && std::strncmp(argv[i + 1], "--", 2) != 0) kv[key] = argv[++i];
            else kv[key] = "1";
        }
    }
    bool has(const char* k) const { return kv.count(k) != 0; }
    std::string str(const char* k, const std::string& d) const {
        auto it = kv.find(k);
        return it == kv.end() ? d : it->second;
    }
    long long i(const char* k, long long d) const {
        auto it = kv.find(k);
        return it == kv.end() ? d : std::atoll(it->second.c_str());
    }
    double f(const char* k, double d) const {
        auto it = kv.find(k);
        return it == kv.end() ? d : std::atof(it->second.c_str());
    }
};

inline void check(bd_status st, const char* what) {
    if (st != BD_OK) {
        std::fprintf(stderr, "%s failed (status %d): %s\n", what, (int)st, bd_last_error_string());
        std::exit(1);
    }
}

inline std::string join(const std::string& dir, const char* name) {
    if (dir.empty() || dir == ".") return name;
    return dir + "/" + name;
}

}  // namespace cli
