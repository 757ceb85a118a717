// The autotuner's cache: the launch shape picked for a batch shape, kept in a
// small JSON file across processes.
//
// Format (one entry per line, written whole by this file only):
//   {
//    "<key>": {"block_threads": 1024, "ctas_per_sm": 1, "rows_per_pass": 2, "cluster_rows": 32768,
//              "cluster_ctas": 16, "clusters": 2, "ms": 61.234},
//    ...
//   }
// A store reads the file, replaces or appends its key and writes the result
// to a temporary file that is renamed over the old one, so a reader never sees
// a half-written file.  Unreadable or malformed lines are dropped; a missing
// file is an empty cache.  Failures are reported, never fatal to a solve.
#include "internal.hpp"

#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace simall {

namespace {

struct Entry {
    std::string key;
    int v[6];
    double ms;
};

bool parse_line(const std::string &line, Entry &e)
{
    const size_t q0 = line.find('"');
    if (q0 == std::string::npos)
        return false;
    const size_t q1 = line.find('"', q0 + 1);
    if (q1 == std::string::npos)
        return false;
    e.key = line.substr(q0 + 1, q1 - q0 - 1);
    const char *rest = line.c_str() + q1 + 1;
    return std::sscanf(rest,
                       " : {\"block_threads\": %d, \"ctas_per_sm\": %d, \"rows_per_pass\": %d, \"cluster_rows\": %d, "
                       "\"cluster_ctas\": %d, \"clusters\": %d, \"ms\": %lf}",
                       &e.v[0], &e.v[1], &e.v[2], &e.v[3], &e.v[4], &e.v[5], &e.ms) == 7;
}

std::vector<Entry> read_entries(const char *path)
{
    std::vector<Entry> out;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        Entry e;
        if (parse_line(line, e))
            out.push_back(e);
    }
    return out;
}

bool key_ok(const char *key)
{
    if (!key || !*key)
        return false;
    for (const char *c = key; *c; ++c)
        if (*c == '"' || *c == '\\' || static_cast<unsigned char>(*c) < 32)
            return false;
    return true;
}

// mkdir -p of the directory part of path.
void make_parent_dirs(const std::string &path)
{
    for (size_t i = 1; i < path.size(); ++i)
        if (path[i] == '/') {
            const std::string d = path.substr(0, i);
            ::mkdir(d.c_str(), 0755);
        }
}

}  // namespace

// SIMALL_AUTOTUNE_CACHE if set ("" or "off": no cache), else
// $XDG_CACHE_HOME/simall_gb300/autotune.json, else
// $HOME/.cache/simall_gb300/autotune.json, else none.
std::string default_autotune_cache_path()
{
    if (const char *p = std::getenv("SIMALL_AUTOTUNE_CACHE"))
        return (std::strcmp(p, "off") == 0) ? std::string() : std::string(p);
    if (const char *x = std::getenv("XDG_CACHE_HOME"); x && *x)
        return std::string(x) + "/simall_gb300/autotune.json";
    if (const char *h = std::getenv("HOME"); h && *h)
        return std::string(h) + "/.cache/simall_gb300/autotune.json";
    return std::string();
}

}  // namespace simall

using namespace simall;

extern "C" {

int simall_autotune_cache_lookup(const char *path, const char *key, int *values)
{
    if (!path || !*path || !key_ok(key) || !values)
        return SIMALL_ERR_INVALID_ARGUMENT;
    for (const Entry &e : read_entries(path))
        if (e.key == key) {
            std::memcpy(values, e.v, sizeof e.v);
            return SIMALL_OK;
        }
    return SIMALL_ERR_IO;
}

int simall_autotune_cache_store(const char *path, const char *key, const int *values, double ms)
{
    if (!path || !*path || !key_ok(key) || !values)
        return SIMALL_ERR_INVALID_ARGUMENT;
    std::vector<Entry> es = read_entries(path);
    bool found = false;
    for (Entry &e : es)
        if (e.key == key) {
            std::memcpy(e.v, values, sizeof e.v);
            e.ms = ms;
            found = true;
        }
    if (!found) {
        Entry e;
        e.key = key;
        std::memcpy(e.v, values, sizeof e.v);
        e.ms = ms;
        es.push_back(e);
    }
    const std::string p(path);
    make_parent_dirs(p);
    const std::string tmp = p + ".tmp." + std::to_string(static_cast<long long>(::getpid()));
    {
        std::ofstream f(tmp, std::ios::trunc);
        if (!f)
            return SIMALL_ERR_IO;
        f << "{\n";
        for (size_t i = 0; i < es.size(); ++i) {
            char buf[192];
            std::snprintf(buf, sizeof buf,
                          "{\"block_threads\": %d, \"ctas_per_sm\": %d, \"rows_per_pass\": %d, \"cluster_rows\": %d, "
                          "\"cluster_ctas\": %d, \"clusters\": %d, \"ms\": %.3f}",
                          es[i].v[0], es[i].v[1], es[i].v[2], es[i].v[3], es[i].v[4], es[i].v[5], es[i].ms);
            f << " \"" << es[i].key << "\": " << buf << (i + 1 < es.size() ? ",\n" : "\n");
        }
        f << "}\n";
        if (!f.good()) {
            std::remove(tmp.c_str());
            return SIMALL_ERR_IO;
        }
    }
    if (std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return SIMALL_ERR_IO;
    }
    return SIMALL_OK;
}

}  // extern "C"
