// ref_wrap.cpp -- extern "C" wrappers around the reference's own element math
// (TEST INFRASTRUCTURE). Compiled by oracle/Makefile against the reference's
// header sources where they lie; output only into oracle/_ref/.
extern "C" int ref_wrap_version() { return 1; }
