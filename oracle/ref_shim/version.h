/* Version strings for the CPU checker build of the reference encoder
 * (the reference generates this file with version.sh; its values only
 * appear in log messages). */
#ifndef XAVS2_VERSION_H
#define XAVS2_VERSION_H
#define VER_MAJOR       1
#define VER_MINOR       4
#define VER_BUILD       0
#define VER_SHA_STR     "checker"
#define _TOSTR(x)       #x
#define TOSTR(x)        _TOSTR(x)
#define XVERSION        VER_MAJOR, VER_MINOR, VER_BUILD
#define XVERSION_STR    TOSTR(VER_MAJOR) "." TOSTR(VER_MINOR) "." TOSTR(VER_BUILD) " " VER_SHA_STR
#define XBUILD_TIME     "checker"
#endif
