// render_main.cpp -- command-line driver for the reference renderer built
// from the pbrt-v2 fork's sources (oracle/ref/Makefile, target pbrt_ref):
// pbrtInit, ParseFile, pbrtCleanup, as main/pbrt.cpp:33-85 does.
// TEST INFRASTRUCTURE ONLY: it renders the reference images the GPU
// renderer is checked against.
#include "stdafx.h"
#include "api.h"
#include "probes.h"
#include "parser.h"
#include "parallel.h"

int main(int argc, char* argv[]) {
    Options options;
    options.quiet = true;
    options.nCores = 0;
    static char path[] = "./";
    options.pbrtPath = path;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "--ncores") && i + 1 < argc) options.nCores = atoi(argv[++i]);
    }
    pbrtInit(options);
    int rc = 0;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "--ncores")) { ++i; continue; }
        if (!ParseFile(argv[i])) { rc = 1; break; }
    }
    pbrtCleanup();
    return rc;
}
