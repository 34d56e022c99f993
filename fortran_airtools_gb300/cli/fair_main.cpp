// fair_main -- drop-in for the reference's main.exe (main.f90) on the GB300
// library: the same flags, defaults, messages and output files, with the
// matrix built and the iterations run through the C-ABI.
//
// main.f90 behaviour kept: at most 9 arguments, each cut to 32 characters
// (flagchar is character(32)); a flag is the first two characters and its
// value the rest; test mode is on from the start (main.f90:55), so -i only
// records the file name; 'rand', 'sym', 'gd', 'sirt' map to 'randkaczmarz',
// 'symkaczmarz', 'graddescent', 'sart'; 'eg'/'twin' and 'ms' map to
// 'errorgauge' and 'mutualstep'; -f switches the stopping rule to the
// oracle; -s and -r together stop; the solution goes to sol.txt (or -o), one
// value per line, and with a stopping rule the error gauge to
// errorgauge.txt. The reference's "stop" messages are printed as
// "STOP <message>" on stderr with exit status 0, as gfortran does.
//
// Added here: -I[inputfile] runs the input-file mode of main.f90:222-271
// (read_data, angle culling by -c, -f reference solution, the grid scaling,
// fanlineartomo, A scaled by grid_size/N, b = -log(T)), which the shipped
// binary never reaches. Phantoms (computed on the GPU): 'shepplogan',
// 'smooth', 'grains', '3phases'; the gallery's others are not part of this
// build. The environment
// variable FAIR_SEED seeds the library's random stream (the reference's
// random_number is unseeded).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fair_gpu.h"
#include "fair_io.h"
#include "fair_phantom.h"

namespace {

// Fortran STOP: a message is printed as "STOP <message>", a bare STOP prints
// nothing; the exit status is 0.
[[noreturn]] void stop(const std::string &msg) {
    fflush(stdout);
    if (!msg.empty()) fprintf(stderr, "STOP %s\n", msg.c_str());
    exit(0);
}

[[noreturn]] void fail(int st, const char *what) {
    fflush(stdout);
    // statuses the reference reports with a STOP (bad sizes, unknown method,
    // a ray outside the grid, the noise generator's Newton iteration)
    if (st == FAIR_ERR_SIZE || st == FAIR_ERR_METHOD || st == FAIR_ERR_GEOMETRY ||
        st == FAIR_ERR_NEWTON)
        stop(fair_error_string(st));
    const char *d = fair_last_error_detail();
    fprintf(stderr, "fair_main: %s: %s%s%s\n", what, fair_error_string(st), d && *d ? " - " : "",
            d ? d : "");
    exit(1);
}

void check(int st, const char *what) {
    if (st != FAIR_OK) fail(st, what);
}

std::string trim(std::string s) {
    size_t a = s.find_first_not_of(' '), b = s.find_last_not_of(' ');
    return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

// READ(str,*) of one item: the first token (blank, comma or slash ends it).
std::string first_token(const std::string &s) {
    size_t a = s.find_first_not_of(" ,");
    if (a == std::string::npos) return "";
    size_t b = s.find_first_of(" ,/", a);
    return s.substr(a, b == std::string::npos ? std::string::npos : b - a);
}

double read_real(const std::string &s, const char *flag) {
    std::string t = first_token(s);
    for (char &c : t)
        if (c == 'd' || c == 'D') c = 'e';
    char *end = nullptr;
    double v = strtod(t.c_str(), &end);
    if (t.empty() || !end || *end) {
        fprintf(stderr, "fair_main: cannot read a number from %s%s\n", flag, s.c_str());
        exit(2);
    }
    return v;
}

int read_int(const std::string &s, const char *flag) {
    std::string t = first_token(s);
    char *end = nullptr;
    long v = strtol(t.c_str(), &end, 10);
    if (t.empty() || !end || *end) {
        fprintf(stderr, "fair_main: cannot read an integer from %s%s\n", flag, s.c_str());
        exit(2);
    }
    return (int)v;
}

bool one_of(const std::string &v, const std::vector<std::string> &set) {
    for (const auto &s : set)
        if (v == s) return true;
    return false;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void help(const std::vector<std::string> &methods) {
    printf(" Main CT AIR tools input flags:\n");
    printf(" -i[inputfile]    Provide suitable inputfile.\n");
    printf(" -o[outputfile]   Choose output file name.\n");
    printf(" -M[method]       Choose which method to use. Standard is Kaczmarz.\n");
    printf("                  Choose from: ");
    for (int j = 0; j < 8; ++j) printf("'%s', ", methods[j].c_str());
    printf("and '%s'.\n", methods[8].c_str());
    printf(" -S[stoprule]     Choose what stopping rule to use. Standard is none.\n");
    printf("                  Choose from 'errorgauge' or 'mutualstep'. Omit if no stopping rule is required.\n");
    printf(" -K[iterations]   Set maximum number of iterations, standard is 100.\n");
    printf(" -O[orderfile]    Ordering of rows, supplied as a list of integers in a file. \n");
    printf(" -L[lowerbound]   Set lower bound.\n");
    printf(" -U[upperbound]   Set upper bound.\n");
    printf(" -R[relaxpar]     Set relaxation parameter.\n");
    printf(" -t[phantom]      Test mode, runs a test phantom. Standard is Shepp-Logan.\n");
    printf("                  Possible inputs: 'shepplogan'.\n");
    printf(" -c[cull]         Cull factor. Only use every cull angles, cull must be an integer.\n");
    printf(" -f[oraclefile]   Read in reference solution. Used as an oracle.\n");
    printf(" -v               Verbose mode.\n");
    printf(" -h               Help.\n");
    printf(" -I[inputfile]    (this build) Run the input-file mode on inputfile.\n");
}

}  // namespace

int main(int argc, char **argv) {
    int skip = 0, max_its = 100;
    bool verbose = false, test_mode = true, stop_rule = false, customord = false;
    bool storematrix = false, readmatrix = false, useoracle = false, input_mode = false;
    double inputnoise = 5e-3;
    std::string outputfile = "sol.txt", inputmethod = "kaczmarz", inputphantom = "shepplogan";
    std::string inputfile, inputstoprule, inputorder, matrixfile, oraclefile;
    const std::vector<std::string> methods = {"kaczmarz", "randkaczmarz", "rand", "symkaczmarz",
                                              "sym", "graddescent", "gd", "cimmino", "sart",
                                              "sirt"};
    const std::vector<std::string> stoprules = {"errorgauge", "mutualstep", "eg", "ms", "twin",
                                                "oracle"};
    const std::vector<std::string> phantoms = {"shepplogan", "", "smooth", "3phases",
                                               "3phasesmooth", "binary", "4phases", "mst",
                                               "grains", "bubbles"};
    fair_opts options;
    check(fair_opts_initialise(&options), "options");
    if (const char *seed = getenv("FAIR_SEED"))  // the library stream's seed (default 0)
        check(fair_random_seed(strtoull(seed, nullptr, 10)), "random_seed");
    std::vector<int32_t> ordering;

    const int cac = argc - 1;
    if (cac == 0) stop("Supply input file or activate test mode.");
    if (cac > 9) stop("Too many input arguments.");
    for (int i = 1; i <= cac; ++i) {
        std::string flagchar = argv[i];
        if (flagchar.size() > 32) flagchar.resize(32);  // character(32)
        flagchar = trim(flagchar);                       // adjustl
        const std::string flag = flagchar.substr(0, 2), val = flagchar.size() > 2 ? flagchar.substr(2) : "";
        if (flag == "-h") {
            help(methods);
            stop("");
        } else if (flag == "-i") {
            inputfile = trim(val);
        } else if (flag == "-I") {
            inputfile = trim(val);
            input_mode = true;
            test_mode = false;
        } else if (flag == "-o") {
            outputfile = trim(val);
        } else if (flag == "-v") {
            printf(" Verbose mode on!\n");
            verbose = true;
            options.verbose = 1;
        } else if (flag == "-t") {
            test_mode = true;
            input_mode = false;
            if (!trim(val).empty()) inputphantom = first_token(val);
            if (!one_of(inputphantom, phantoms)) stop("Not a recognised phantom in -t. Use -h for help.");
            if (inputphantom.empty()) inputphantom = "shepplogan";
            printf(" Test mode active. Ignoring input file.\n");
        } else if (flag == "-K") {
            max_its = read_int(val, "-K");
        } else if (flag == "-c") {
            skip = read_int(val, "-c");
        } else if (flag == "-M") {
            inputmethod = first_token(val);
            if (!one_of(inputmethod, methods)) stop("Not a recognised stopping rule. Use -h for help.");
            if (inputmethod == "rand") inputmethod = "randkaczmarz";
            if (inputmethod == "sym") inputmethod = "symkaczmarz";
            if (inputmethod == "gd") inputmethod = "graddescent";
            if (inputmethod == "sirt") inputmethod = "sart";
        } else if (flag == "-n") {
            inputnoise = read_real(val, "-n");
            if (inputnoise < 0) stop("Provide positive noise level.");
        } else if (flag == "-S") {
            stop_rule = true;
            inputstoprule = first_token(val);
            if (!one_of(inputstoprule, stoprules))
                stop("Not a recognised stopping rule. Choose from 'errorgauge' or 'mutualstep'.");
            if (inputstoprule == "eg" || inputstoprule == "twin") inputstoprule = "errorgauge";
            if (inputstoprule == "ms") inputstoprule = "mutualstep";
        } else if (flag == "-L") {
            check(fair_opts_set_lbound(&options, read_real(val, "-L")), "options");
        } else if (flag == "-U") {
            check(fair_opts_set_ubound(&options, read_real(val, "-U")), "options");
        } else if (flag == "-R") {
            options.relaxpar = read_real(val, "-R");
        } else if (flag == "-O") {
            inputorder = first_token(val);
            customord = true;
            if (verbose) printf(" Reading custom ordering.\n");
            int32_t len = 0;
            check(fair_read_ordering(inputorder.c_str(), &len, nullptr, 0), "read_ordering");
            ordering.resize(len > 0 ? len : 1);
            check(fair_read_ordering(inputorder.c_str(), &len, ordering.data(), len), "read_ordering");
            ordering.resize(len);
        } else if (flag == "-r") {
            matrixfile = first_token(val);
            readmatrix = true;
        } else if (flag == "-s") {
            matrixfile = first_token(val);
            storematrix = true;
        } else if (flag == "-f") {
            oraclefile = first_token(val);
            useoracle = true;
        } else if (flag == "-H") {
            printf(" Oh noes, the hamster! RUN!!!\n");
            stop("");
        } else {
            stop("Not a recognised flag, use -h for help.");
        }
    }
    if (useoracle && inputstoprule != "oracle") {
        printf(" Overriding stopping rule. Using oracle instead.\n");
        inputstoprule = "oracle";
        stop_rule = true;
    }
    if (storematrix && readmatrix) stop("Choose either storing or reading matrix.");
    (void)input_mode;

    // ---------------------------------------------------------------- set-up ----
    fair_csr A = nullptr;
    check(fair_csr_create(&A), "fair_csr_create");
    fair_data dat{};
    std::vector<double> theta, xref, b, bt;
    double t0 = 0, t1 = 0;
    if (test_mode) {  // main.f90:190-220
        dat.n = 256;
        dat.nth = 400;
        dat.p = (int32_t)(1.5 * dat.n);
        dat.r = sqrt(2.0);
        dat.dw = 1.0;
        dat.sd = 1.0;
        theta.resize(dat.nth);
        check(fair_linspace(0.0, 3.141592653589793, dat.nth, theta.data()), "linspace");
        dat.theta = theta.data();
        t0 = now_s();
        if (readmatrix) {
            check(fair_read_csr_matrix(A, matrixfile.c_str()), "read_csr_matrix");
        } else {
            if (verbose) printf(" Constructing matrix...\n");
            check(fair_paralleltomo(&dat, A), "paralleltomo");
        }
        if (!one_of(inputphantom, {"shepplogan", "smooth", "grains", "3phases"}))
            stop("Phantom " + inputphantom + " is not part of this build; use 'shepplogan', "
                 "'smooth', 'grains' or '3phases'.");
        const int64_t npix = (int64_t)dat.n * dat.n;
        xref.resize(npix);
        check(fair_phantom(inputphantom.c_str(), dat.n, xref.data()), "choose_phantom");
        int32_t m, n;
        int64_t nnz;
        check(fair_csr_info(A, &m, &n, &nnz), "info");
        if (n != npix) stop("Vector input size incorrect.");
        b.resize(m);
        bt.resize(m);
        std::vector<double> noise(m);
        check(fair_matvecmul(A, xref.data(), npix, b.data()), "matvecmul");
        check(fair_add_white_noise(bt.data(), noise.data(), b.data(), m, inputnoise), "add_white_noise");
        t1 = now_s();
    } else {  // main.f90:222-271, reached here through -I
        if (verbose) printf(" Reading in data...\n");
        int32_t n, p, nth;
        check(fair_read_data_sizes(inputfile.c_str(), &n, &p, &nth), "read_data");
        theta.resize(nth > 0 ? nth : 1);
        std::vector<double> T((size_t)nth * p + 1);
        check(fair_read_data(inputfile.c_str(), &dat, theta.data(), T.data()), "read_data");
        if (verbose) printf(" done.\n");
        if (skip > 0) {  // keep every skip-th angle and its data column
            if (verbose) printf(" Culling data...\n");
            std::vector<double> th2, T2;
            for (int i = 0; i < dat.nth; i += skip) {
                th2.push_back(theta[i]);
                T2.insert(T2.end(), T.begin() + (size_t)i * dat.p, T.begin() + (size_t)(i + 1) * dat.p);
            }
            theta = th2;
            T = T2;
            dat.nth = (int32_t)theta.size();
            dat.theta = theta.data();
            if (verbose) printf(" done.\n");
        }
        if (useoracle) {
            xref.resize((size_t)dat.n * dat.n);
            check(fair_read_ref(oraclefile.c_str(), (int64_t)dat.n * dat.n, xref.data()), "read_ref");
        }
        t0 = now_s();
        const double grid_size = dat.dw * dat.r / dat.sd;  // main.f90:248-252
        dat.r = dat.r / grid_size;
        dat.dw = dat.dw / grid_size;
        dat.sd = dat.sd / grid_size;
        if (readmatrix) {
            check(fair_read_csr_matrix(A, matrixfile.c_str()), "read_csr_matrix");
        } else {
            if (verbose) printf(" Constructing matrix...\n");
            check(fair_fanlineartomo(&dat, 0, A), "fanlineartomo");
            check(fair_multiply_by_scalar(A, grid_size / dat.n), "multiply_by_scalar");
        }
        int32_t m, nn;
        int64_t nnz;
        check(fair_csr_info(A, &m, &nn, &nnz), "info");
        if ((int64_t)m > (int64_t)T.size()) stop("Vector input size incorrect.");
        bt.resize(m);
        for (int32_t k = 0; k < m; ++k) bt[k] = -log(T[k]);
        t1 = now_s();
    }
    if (storematrix) check(fair_store_matrix(A, matrixfile.c_str()), "store_matrix");
    int32_t m, n;
    int64_t nnz;
    check(fair_csr_info(A, &m, &n, &nnz), "info");
    if (verbose) {
        printf(" done in %14.7f  seconds!\n", t1 - t0);
        printf("  \n");
        printf(" Matrix size: %11d  by %11d\n", m, n);
        printf(" nnz: %11lld\n", (long long)nnz);
        printf(" sparsity level: %25.17f\n", (1.0 * nnz) / (1.0 * m * n));
        printf(" space saved: %25.17f %%\n", (1.0 - (2.0 * nnz + m + 1) / (1.0 * m * n)) * 100.0);
        printf("  \n");
        if (test_mode) printf(" Noise level: %25.17f\n", inputnoise);
    }

    // ------------------------------------------------------------- execution ----
    t0 = now_s();
    const int64_t npix = (int64_t)dat.n * dat.n;
    std::vector<double> EG(max_its > 0 ? max_its : 1, 0.0), xout(npix > n ? npix : n, 0.0);
    std::vector<double> Xstore(xout.size()), Ystore(xout.size());
    const int32_t Kin = max_its;
    const int32_t *ord = customord ? ordering.data() : nullptr;
    const int32_t nord = customord ? (int32_t)ordering.size() : 0;
    if (inputmethod == "graddescent") {
        check(fair_gradient_descent(xout.data(), A, bt.data(), &Kin, nullptr, nullptr, nullptr,
                                    &options, nullptr), "gradient_descent");
    } else if (inputmethod == "cimmino" || inputmethod == "sart") {
        check(fair_sirt(xout.data(), inputmethod.c_str(), A, bt.data(), &Kin, 1, nullptr, &options),
              "sirt");
    } else if (stop_rule && inputstoprule == "oracle") {
        if (xref.empty()) stop("An oracle needs a reference solution (-f).");
        check(fair_art(Xstore.data(), inputmethod.c_str(), A, bt.data(), &Kin, 1, nullptr,
                       xref.data(), ord, nord, &options), "art");
        xout = Xstore;
    } else if (stop_rule) {
        int32_t final_it = 0;
        check(fair_twin_art(xout.data(), &final_it, Xstore.data(), Ystore.data(), EG.data(),
                            inputmethod.c_str(), inputstoprule.c_str(), A, bt.data(), &Kin, 1,
                            nullptr, nullptr, ord, nord, -1, &options), "twin_art");
    } else {
        check(fair_art(Xstore.data(), inputmethod.c_str(), A, bt.data(), &Kin, 1, nullptr, nullptr,
                       ord, nord, &options), "art");
        xout = Xstore;
    }
    if (verbose && test_mode) {
        double num = 0, den = 0;
        for (int64_t k = 0; k < npix; ++k) {
            num += (xref[k] - xout[k]) * (xref[k] - xout[k]);
            den += xref[k] * xref[k];
        }
        printf(" Final error: %25.17f\n", sqrt(num) / sqrt(den));
    }
    t1 = now_s();
    if (verbose) printf(" Done in %14.7f  seconds.\n", t1 - t0);

    // ------------------------------------------------------------------ output ----
    check(fair_write_values(outputfile.c_str(), xout.data(), n), "write solution");
    if (stop_rule) check(fair_write_values("errorgauge.txt", EG.data(), max_its), "write error gauge");
    fair_csr_destroy(A);
    return 0;
}
