// cli.cpp -- the `cluster` executable: same arguments and output file as the
// reference's ./cluster (cuda-version/main.cu).
#include "gsdr.h"

int main(int argc, char** argv) { return gsdr_main(argc, argv); }
