// ses3d-nt-gpu CONFIG [--fp64]: the forward workflow of the ses3d-nt driver
// (src/ses3d-nt.F90, workflow 'forward') with the time step on the GPU.
// Reads the NAMELIST config and its raw model files, writes one SAC trace per
// receiver channel. Exit status 0 on success, 1 on error (message on stderr).
#include <cstdio>
#include <cstring>

#include "../../include/sesnt.h"

int main(int argc, char **argv) {
    if (argc < 2 || std::strcmp(argv[1], "-h") == 0 || std::strcmp(argv[1], "--help") == 0) {
        std::fprintf(stderr, "usage: %s CONFIG [--fp64]\n", argv[0]);
        return argc < 2 ? 1 : 0;
    }
    const int precision = (argc > 2 && std::strcmp(argv[2], "--fp64") == 0) ? 8 : 4;
    int traces = 0;
    const int rc = sesnt_forward(argv[1], precision, &traces);
    if (rc != SESNT_OK) {
        std::fprintf(stderr, "ses3d-nt-gpu: error %d: %s\n", rc, sesnt_config_last_error());
        return 1;
    }
    std::printf("ses3d-nt-gpu: %d SAC traces written\n", traces);
    return 0;
}
