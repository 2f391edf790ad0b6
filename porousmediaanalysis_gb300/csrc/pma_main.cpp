// pma command-line tool: the same modes as the reference executable
// (CommandLineDispatcher.cpp:123-154, Main.cpp:30-99). Runs the selected mode on every
// folder under the current working directory that holds a config.txt.
#include <unistd.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/pma.h"

static void usage() {
    std::printf(
        "Console parameters are incorrect. Exiting.\n\n"
        "The following console parameters are supported:\n"
        "-edt - calculates Euclidean distance transform (maximum inscribed balls)\n"
        "-rib - removes inner balls (balls fully contained in other balls)\n"
        "-apt - assigns pores and throats\n"
        "-all - determines maximum inscribed balls, medial axis, pores, throats, and pore connectivity statistics\n"
        "-spd - computes shortest path distances (requires only initial binary image)\n");
}

int main(int argc, char** argv) {
    setvbuf(stdout, nullptr, _IONBF, 0);  // Main.cpp:35
    pma_mode mode;
    if (argc < 2) {
        usage();
        return 0;
    }
    const std::string a = argv[1];
    if (a == "-all") mode = PMA_MODE_ALL;
    else if (a == "-edt") mode = PMA_MODE_EDT;
    else if (a == "-rib") mode = PMA_MODE_RIB;
    else if (a == "-apt") mode = PMA_MODE_APT;
    else if (a == "-spd") mode = PMA_MODE_SPD;
    else {
        usage();
        return 0;
    }
    // "--strict" turns errors into a non-zero exit code; the reference always exits 0.
    bool strict = argc > 2 && std::strcmp(argv[2], "--strict") == 0;
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) {
        std::printf("cannot read the working directory\n");
        return strict ? 1 : 0;
    }
    pma_ctx* ctx = nullptr;
    int rc = pma_ctx_create(0, &ctx);
    if (rc == PMA_OK) rc = pma_run_folder(ctx, cwd, mode);
    if (rc != PMA_OK) {
        char msg[2048];
        pma_last_error(msg, sizeof(msg));
        std::printf("%s\n", msg);
    }
    pma_ctx_destroy(ctx);
    return (strict && rc != PMA_OK) ? 1 : 0;
}
