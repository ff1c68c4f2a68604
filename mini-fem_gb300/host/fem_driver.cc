// minifem_fem — the reference driver's flow (src/main.cc:96-388 and the
// FEM loop of src/FEM.cc:139-285) at one rank, calling the drop-in operators of
// operators_gpu.cc.  It exists so that the drop-in can be run end to end where
// the reference sources are not available:
//
//   MINIFEM_DATA_PATH=<root> minifem_fem <mesh> <lap|ela> <iterations>
//
// reads <root>/<mesh>/inputs/<op>_1_0 (layout of src/IO.cc:61-96), optionally
// colours and permutes the elements in place (MINIFEM_COLORING=1, as the
// COLORING build does at src/main.cc:209-236), builds the CSR from the
// node -> element lists (src/main.cc:238-250), optionally the element -> CSR
// position map (MINIFEM_OPTIMIZED=1, as the OPTIMIZED build does at
// src/main.cc:319-333), the Dirichlet mask, runs the
// iterations (iteration 0 untimed when there are several, src/FEM.cc:182) and
// prints the relative norm differences against <root>/<mesh>/checkings/<op>_1_0
// (src/FEM.cc:59-98).
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "minifem_dropin.h"

int *colorToElem = nullptr;
int nbTotalColors = 0;

namespace {

struct Timer {
    uint64_t total = 0, count = 0;
    std::chrono::steady_clock::time_point t0;
    void start() { t0 = std::chrono::steady_clock::now(); }
    void stop() {
        total += std::chrono::duration_cast<std::chrono::nanoseconds>(
                     std::chrono::steady_clock::now() - t0).count();
        count++;
    }
    uint64_t avg() const { return count ? total / count : 0; }
};

double norm2(const double *x, long n) {
    double s = 0;
    for (long i = 0; i < n; i++) s += x[i] * x[i];
    return std::sqrt(s);
}

[[noreturn]] void fail(const std::string &m) {
    std::cerr << "Error: " << m << "\n";
    exit(EXIT_FAILURE);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) fail("usage: minifem_fem <mesh> <lap|ela> <iterations>");
    const std::string mesh = argv[1], op = argv[2];
    const int nbIter = (int)strtol(argv[3], nullptr, 0);
    if (op != "lap" && op != "ela") fail("operator must be lap or ela");
    if (nbIter < 1) fail("Number of iterations must be at least 1.");
    const int operatorDim = op == "lap" ? 1 : 9, operatorID = op == "lap" ? 0 : 1;
    const char *root = getenv("MINIFEM_DATA_PATH");
    const std::string base = std::string(root ? root : ".") + "/" + mesh;

    std::ifstream in(base + "/inputs/" + op + "_1_0", std::ios::binary);
    if (!in) fail("cannot read input data: " + base + "/inputs/" + op + "_1_0");
    int hdr[6];
    in.read((char *)hdr, sizeof(hdr));
    const int nbElem = hdr[0], nbNodes = hdr[1], nbEdges = hdr[2], nbIntf = hdr[3],
              nbIntfNodes = hdr[4], nbBound = hdr[5];
    std::vector<double> coord((size_t)nbNodes * 3);
    std::vector<int> e2n((size_t)nbElem * 4), skip((size_t)std::max(nbIntf, 1) * 3 + nbIntf + 1 + nbIntfNodes),
        code(nbNodes);
    in.read((char *)coord.data(), coord.size() * sizeof(double));
    in.read((char *)e2n.data(), e2n.size() * sizeof(int));
    in.read((char *)skip.data(), skip.size() * sizeof(int));
    in.read((char *)code.data(), code.size() * sizeof(int));
    if (!in) fail("truncated input data");

    std::cout << "\t\t* Mini-FEM (GB300 operators) *\n\nTest case : \"" << mesh
              << "\"\nOperator  : \"" << op << "\"\nIterations:  " << nbIter << "\n\n";

    if (getenv("MINIFEM_COLORING") && atoi(getenv("MINIFEM_COLORING"))) {
        std::vector<int> perm(nbElem), tmp(e2n);
        coloring_creation(e2n.data(), perm.data(), nbElem, nbNodes);
        for (int e = 0; e < nbElem; e++)
            std::memcpy(&e2n[(size_t)perm[e] * 4], &tmp[(size_t)e * 4], 4 * sizeof(int));
        std::cout << "Colours                : " << nbTotalColors << "\n";
    }

    // CSR: the caller builds the node -> element index the way src/main.cc:243-247 does
    index_t nodeToElem;
    std::vector<int> nteIndex(nbNodes + 1, 0), nteValue((size_t)nbElem * 4);
    for (int v : e2n) nteIndex[v]++;
    for (int i = 0; i < nbNodes; i++) nteIndex[i + 1] += nteIndex[i];
    {
        std::vector<int> fill(nbNodes, 0);
        for (int e = 0; e < nbElem; e++)
            for (int k = 0; k < 4; k++) {
                int n = e2n[(size_t)e * 4 + k] - 1;
                nteValue[nteIndex[n] + fill[n]++] = e;
            }
    }
    nodeToElem.index = nteIndex.data();
    nodeToElem.value = nteValue.data();
    std::vector<int> row(nbNodes + 1), col(nbEdges);
    create_nodeToNode(row.data(), col.data(), nodeToElem, e2n.data(), nbNodes);
    if (row[nbNodes] != nbEdges) fail("nbEdges of the mesh file differs from the CSR size");

    std::vector<int> elemToEdge;
    if (getenv("MINIFEM_OPTIMIZED") && atoi(getenv("MINIFEM_OPTIMIZED"))) {
        elemToEdge.resize((size_t)nbElem * 16);
        create_elemToEdge(row.data(), col.data(), e2n.data(), elemToEdge.data(), nbElem);
        std::cout << "Edges index            : " << elemToEdge.size() << " positions\n";
    }

    // Dirichlet mask: boundary list (src/Fortran/qdmrd4.f) then per-DOF flags
    // (src/Fortran/e_cgmelissa.F: codes 52/53/54 fix x/y/z, other codes fix all)
    std::vector<int> checkBounds((size_t)nbNodes * 3, 0);
    int listed = 0;
    for (int i = 0; i < nbNodes; i++) {
        if (code[i] == 0) continue;
        listed++;
        if (code[i] == 52) checkBounds[i] = 1;
        else if (code[i] == 53) checkBounds[i + (size_t)nbNodes] = 1;
        else if (code[i] == 54) checkBounds[i + 2 * (size_t)nbNodes] = 1;
        else checkBounds[i] = checkBounds[i + (size_t)nbNodes] = checkBounds[i + 2 * (size_t)nbNodes] = 1;
    }
    if (listed > nbBound) fail("more boundary nodes than nbBoundNodes");

    std::vector<double> values((size_t)nbEdges * operatorDim), prec((size_t)nbNodes * operatorDim);
    Timer asmT, initT, invT;
    for (int iter = 0; iter < nbIter; iter++) {
        const bool timed = nbIter == 1 || iter > 0;
        if (timed) asmT.start();
        assembly(coord.data(), values.data(), row.data(), col.data(), e2n.data(),
                 elemToEdge.empty() ? nullptr : elemToEdge.data(), nbElem, nbEdges, operatorDim,
                 operatorID);
        if (timed) asmT.stop();
        if (timed) initT.start();
        prec_init(prec.data(), values.data(), row.data(), col.data(), nbNodes, operatorDim);
        if (timed) initT.stop();
        if (timed) invT.start();
        prec_inversion(prec.data(), row.data(), col.data(), checkBounds.data(), nbNodes, operatorID);
        if (timed) invT.stop();
    }
    std::cout << "Average time (ns)\n----------------------------------------------\n"
              << "  Matrix assembly               : " << asmT.avg() << "\n"
              << "  Preconditioner initialization : " << initT.avg() << "\n"
              << "  Halo exchange                 : 0\n"
              << "  Preconditioner inversion      : " << invT.avg() << "\n"
              << "  Total                         : " << asmT.avg() + initT.avg() + invT.avg()
              << "\n----------------------------------------------\n\n";

    const double mn = norm2(values.data(), (long)values.size()), pn = norm2(prec.data(), (long)prec.size());
    std::ifstream chk(base + "/checkings/" + op + "_1_0");
    if (!chk) fail("cannot read reference checking: " + base + "/checkings/" + op + "_1_0");
    double refM = 0, refP = 0;
    chk >> refM >> refP;
    std::cout << std::scientific << std::setprecision(1)
              << "Numerical stability of rank 0\n----------------------------------------------\n"
              << "  Matrix -> reference norm : " << refM << "\n"
              << "              current norm : " << mn << "\n"
              << "                difference : " << std::abs(refM - mn) / refM << "\n\n"
              << "    Prec -> reference norm : " << refP << "\n"
              << "              current norm : " << pn << "\n"
              << "                difference : " << std::abs(refP - pn) / refP << "\n"
              << "----------------------------------------------\n";
    delete[] colorToElem;
    return EXIT_SUCCESS;
}
