// blamm_main.cpp -- the `blamm` command line (blstools.cpp:113-166): dict, hist, scan.
#include <iostream>
#include <stdexcept>
#include <string>

#include "blamm_gpu.h"
#include "histogram.h"
#include "species.h"

namespace blamm {
int runScanModule(int argc, char **argv);
}

static void printUsage()
{
    std::cout << "Usage: blamm command [options]\n\n"
                 " command\n"
                 "  dict\t\t\tmake a dictionary for the input sequences\n"
                 "  hist\t\t\tgenerate PWM score histograms\n"
                 "  scan\t\t\tscan for pwm occurrences\n\n"
                 " [options]\n"
                 "  -h\t--help\t\tdisplay help page\n"
                 "  -v\t--version\tdisplay version\n\n";
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        printUsage();
        return EXIT_FAILURE;
    }
    const std::string cmd(argv[1]);
    if (cmd == "-h" || cmd == "--help") {
        printUsage();
        return EXIT_SUCCESS;
    }
    if (cmd == "-v" || cmd == "--version") {
        const int v = blamm_version();
        std::cout << "BLAS Accelerated Motif Matching (blamm) -- GB300 build, library version " << v / 10000
                  << "." << (v / 100) % 100 << "." << v % 100 << "\n";
        return EXIT_SUCCESS;
    }
    try {
        if (cmd == "dict") blamm::runDictModule(argc, argv);
        else if (cmd == "hist") blamm::runHistModule(argc, argv);
        else if (cmd == "scan") {
            if (blamm::runScanModule(argc, argv) != 0) return EXIT_FAILURE;
        } else {
            printUsage();
            return EXIT_FAILURE;
        }
    } catch (std::exception &e) {
        // the reference's run*Module: message on stderr, EXIT_FAILURE (blstools.cpp:63-101)
        std::cerr << e.what() << std::endl;
        return EXIT_FAILURE;
    }
    std::cout << "Exiting... bye!" << std::endl;
    return EXIT_SUCCESS;
}
