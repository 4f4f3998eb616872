// latticegen: command-line drop-in for the reference lattice generator
// (Source code/latticegen2_W8/main.cpp:19-71):
//   latticegen <geometry> <nodes in x> <xseed> <yseed> <zseed> <output> <1|2>
// reads STARCDfiles/<geometry>.vrt and .bnd, writes <output>_Node.dat and
// <output>_BC.dat.
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

#include <string>

extern "C" int lbm_latticegen(const char *vrt_path, const char *bnd_path, int n_x, double xseed,
                              double yseed, double zseed, int complexity, const char *node_path,
                              const char *bc_path, int *out_dims);
extern "C" const char *lbm_latticegen_error(void);

int main(int argc, char **argv) {
    if (argc != 8) {
        printf("Usage: latticegen <input_filename> <NoOfNodes in X dir> <xseed> <yseed> <zseed> "
               "<output filename> <1- simple, 2 - complex geometry>\n");
        return 1;
    }
    const clock_t t0 = clock();
    const std::string geo = std::string("STARCDfiles/") + argv[1];
    const std::string out = argv[6];
    int dims[3] = {0, 0, 0};
    const int rc = lbm_latticegen((geo + ".vrt").c_str(), (geo + ".bnd").c_str(), atoi(argv[2]),
                                  atof(argv[3]), atof(argv[4]), atof(argv[5]), atoi(argv[7]),
                                  (out + "_Node.dat").c_str(), (out + "_BC.dat").c_str(), dims);
    if (rc != 0) {
        fprintf(stderr, "latticegen: %s\n", lbm_latticegen_error());
        return rc;
    }
    printf("lattice %d x %d x %d written to %s_Node.dat / %s_BC.dat in %.2fs\n", dims[0], dims[1],
           dims[2], out.c_str(), out.c_str(), (double)(clock() - t0) / CLOCKS_PER_SEC);
    return 0;
}
