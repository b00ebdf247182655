/* Test-infrastructure stub (oracle build only): the few MSVC CRT names the
 * reference's utils.hxx uses (_splitpath_s, _MAX_* limits, errno_t). */
#pragma once
#include <cstring>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <string>
#include <fstream>
#include <sstream>
#include <iomanip>
#include <deque>
#include <map>
#include <list>
#include <memory>
#include <typeinfo>
typedef int errno_t;
#ifndef _MAX_DRIVE
#define _MAX_DRIVE 3
#define _MAX_DIR 256
#define _MAX_FNAME 256
#define _MAX_EXT 256
#endif
static inline errno_t _splitpath_s(const char *path, char *drive, size_t dn, char *dir, size_t dirn,
                                   char *fname, size_t fn, char *ext, size_t en)
{
    std::string p(path ? path : "");
    std::string d, f, e;
    size_t slash = p.find_last_of("/\\");
    if (slash != std::string::npos) { d = p.substr(0, slash + 1); p = p.substr(slash + 1); }
    size_t dot = p.find_last_of('.');
    if (dot != std::string::npos) { e = p.substr(dot); f = p.substr(0, dot); } else f = p;
    if (drive && dn) drive[0] = 0;
    if (dir && dirn) { std::strncpy(dir, d.c_str(), dirn - 1); dir[dirn - 1] = 0; }
    if (fname && fn) { std::strncpy(fname, f.c_str(), fn - 1); fname[fn - 1] = 0; }
    if (ext && en) { std::strncpy(ext, e.c_str(), en - 1); ext[en - 1] = 0; }
    return 0;
}
