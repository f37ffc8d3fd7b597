// Shared helpers of the command-line drop-ins (timers, form selection).
#pragma once
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include <string>

#include "../../include/parent_gb300.h"

static inline double wall_seconds() {
    timeval tv;
    gettimeofday(&tv, nullptr);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

// Last '.'-separated token of a file name, as the reference's strtok loop
// (PARENT.cpp:196-206) extracts the extension.
static inline std::string last_ext(const char *path) {
    std::string s(path);
    size_t p = s.find_last_of('.');
    return p == std::string::npos ? s : s.substr(p + 1);
}

// GPU options the reference does not read: PG_DEVICE (default 0) and
// PG_FORM = auto | hist | onehot (default auto).
static inline int env_device() {
    const char *e = getenv("PG_DEVICE");
    return e ? atoi(e) : 0;
}
static inline int env_form() {
    const char *e = getenv("PG_FORM");
    if (!e || !strcmp(e, "auto")) return PG_FORM_AUTO;
    if (!strcmp(e, "hist")) return PG_FORM_HIST;
    if (!strcmp(e, "onehot")) return PG_FORM_ONEHOT;
    return -1;
}
