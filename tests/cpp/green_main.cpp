// A compiled C++ caller of the drop-in entry point, written like the
// reference's own test executable (cusrc/main.cu:1-10): it includes the
// library's header in place of popm/popm.h and calls
//     green("../cusrc/example/crust1.0.txt", "out4.txt", "signal.txt");
// with the same string literals, so the reference's caller compiles and links
// against libgrtm_gb300.so unchanged.  Given three arguments it calls green()
// with them instead (input file, spectra file, time-series file).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "grtm_gb300.h"

int main(int argc, char **argv)
{
    if (argc == 4) {
        green(argv[1], argv[2], argv[3]);
        return 0;
    }
    green("../cusrc/example/crust1.0.txt", "out4.txt", "signal.txt");
    return 0;
}
