// nanofiller.cpp -- command-line front end over the C ABI, with the verb syntax
// of the reference's NanoFiller binary (src/NanoFiller.cpp:37-162):
//
//   nanofiller <parameter file> [generate] [verb ...]
//
// `generate` draws the rods (nf_generate; output.bin is written when WRT_BIN is
// set); without it the rods are read from output.bin in the working directory.
// Verbs on this path:
//   write_vtk             output.vtk (write_CNTvtk layout)
//   expand <dir>          field axis of the electrodes (1 = x, 2 = y, 4 = z); the
//                         electrodes are the two faces of that axis
//   stat_conduct <dir>    contacts with screening and electrode roles, written as
//                         internal.srt.coo, sink.elec.coo, source.elec.coo, then
//                         the network solve (G_eff printed)
//   stat_conduct <dir> internal
//                         the same with the intra-rod resistor network: nodes at
//                         the contact points, rod segments between them, written
//                         as Nodes.tbl.dat, segment.LA.coo, internal.DS.coo,
//                         sink.DS.coo, source.DS.coo, then the node-network solve
//   reduce <dir>          dead-end pruning: rods with fewer than 2 contacts
//                         within STAT_DIST_LIM (unscreened, electrodes count)
//                         are removed until none is; reduced.bin with WRT_BIN 1
//   stat_nematic          nematic order parameter about z, printed
//   stat_phitheta         32 x 32 histogram of rod directions, rho.dat
//   stat_mutangle         32-bin histogram of mutual angles of contacting rods
//                         (closest points interior to both), gamma.dat
//   stat_contacts         contacts per rod within STAT_DIST_LIM: total, mean, max
//   write_ort             rod directions as VTK points, orient.vtk
//   write_lmp             LAMMPS ellipsoid data, output.lmp.data
// The reference's other verbs (plot, stat_exclsurf, stat_vdw) are not part of
// this path: they are reported and the program exits with
// status 2 before any work. Every error exits non-zero with the library's
// message.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "nanofiller_gb300.h"

namespace {

const double kPi = 3.14159265358979323846;

int fail(nf_handle* h, nf_status s, const char* what) {
    char msg[512] = "";
    if (h) nf_last_error(h, msg, sizeof msg);
    std::fprintf(stderr, "nanofiller: %s: %s%s%s\n", what, nf_status_string(s), msg[0] ? ": " : "", msg);
    return 1;
}

struct Verb {
    std::string name;
    int dir;
    bool internal;
};

bool not_on_path(const std::string& v) {
    static const char* other[] = {"plot", "stat_exclsurf", "stat_vdw"};
    for (const char* o : other)
        if (v == o) return true;
    return false;
}

int parse_dir(const char* s, int* dir) {
    char* end = nullptr;
    long d = std::strtol(s, &end, 10);
    if (!end || *end || (d != 1 && d != 2 && d != 4)) return 0;
    *dir = (int)d;
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr,
                     "usage: nanofiller <parameter file> [generate] [write_vtk] [expand <dir>] "
                     "[stat_conduct <dir>]\n");
        return 1;
    }
    // Verbs first, so that a command line this path cannot run does no work.
    bool generate = std::strcmp(argv[2], "generate") == 0;
    std::vector<Verb> verbs;
    int field_dir = 0;
    for (int a = generate ? 3 : 2; a < argc; ++a) {
        std::string v = argv[a];
        if (v == "write_vtk" || v == "stat_nematic" || v == "stat_phitheta" || v == "stat_mutangle" ||
            v == "stat_contacts" || v == "write_ort" || v == "write_lmp") {
            verbs.push_back({v, 0, false});
        } else if (v == "expand" || v == "stat_conduct" || v == "reduce") {
            int d = 0;
            if (a + 1 >= argc || !parse_dir(argv[a + 1], &d)) {
                std::fprintf(stderr, "nanofiller: %s needs a direction 1, 2 or 4\n", v.c_str());
                return 1;
            }
            ++a;
            bool internal = false;
            if (v == "stat_conduct" && a + 1 < argc && std::strcmp(argv[a + 1], "internal") == 0) {
                internal = true;
                ++a;
            }
            if (field_dir && field_dir != d) {
                std::fprintf(stderr, "nanofiller: conflicting directions %d and %d\n", field_dir, d);
                return 1;
            }
            field_dir = d;
            verbs.push_back({v, d, internal});
        } else if (not_on_path(v)) {
            std::fprintf(stderr, "nanofiller: verb '%s' is not part of this path\n", v.c_str());
            return 2;
        } else {
            std::fprintf(stderr, "nanofiller: unknown verb '%s'\n", v.c_str());
            return 1;
        }
    }

    nf_params p;
    nf_params_default(&p);
    int unknown = 0;
    nf_status s = nf_params_from_file(argv[1], &p, &unknown);
    if (s != NF_OK) return fail(nullptr, s, argv[1]);
    if (unknown) std::fprintf(stderr, "nanofiller: %d unknown key(s) in %s ignored\n", unknown, argv[1]);
    if (field_dir) p.field_dir = field_dir;

    nf_handle* h = nullptr;
    s = nf_create(&p, &h);
    if (s != NF_OK) return fail(nullptr, s, "nf_create");
    int rc = 0;
    if (generate) {
        nf_gen_stats g;
        s = nf_generate(h, &g);
        if (s != NF_OK) { rc = fail(h, s, "generate"); goto done; }
        std::printf("%llu inclusions generated from %llu candidates in %.3f ms\n",
                    (unsigned long long)g.accepted, (unsigned long long)g.candidates_drawn, g.ms);
        if (p.wrt_bin) {
            s = nf_write_state_bin(h, "output.bin");
            if (s != NF_OK) { rc = fail(h, s, "output.bin"); goto done; }
        }
    } else {
        s = nf_read_state_bin(h, "output.bin");
        if (s != NF_OK) { rc = fail(h, s, "output.bin"); goto done; }
    }
    {
        // Volume fraction of the rods as cylinders without caps (get_VolFrac,
        // src/simPrms.cpp:1026-1030).
        nf_rods r;
        std::memset(&r, 0, sizeof r);
        s = nf_get_rods(h, &r);
        if (s != NF_OK && s != NF_ERR_CAPACITY) { rc = fail(h, s, "rods"); goto done; }
        std::vector<float> l(r.count), a(r.count);
        r.capacity = r.count;
        r.l = l.data();
        r.a = a.data();
        s = nf_get_rods(h, &r);
        if (s != NF_OK) { rc = fail(h, s, "rods"); goto done; }
        double vol = 0;
        for (size_t i = 0; i < r.count; ++i) vol += kPi * (double)a[i] * a[i] * l[i];
        std::printf("Volume fraction of %5.2f percent is achieved\n",
                    100.0 * vol / ((double)p.box[0] * p.box[1] * p.box[2]));
    }
    for (const Verb& v : verbs) {
        if (v.name == "write_vtk") {
            s = nf_write_vtk(h, "output.vtk");
            if (s != NF_OK) { rc = fail(h, s, "write_vtk"); goto done; }
        } else if (v.name == "stat_nematic") {
            const double z[3] = {0.0, 0.0, 1.0};
            double S = 0;
            s = nf_stat_nematic(h, z, &S);
            if (s != NF_OK) { rc = fail(h, s, "stat_nematic"); goto done; }
            std::printf("Estimated nematic order parameter: %f\n", S);
        } else if (v.name == "stat_phitheta") {
            std::vector<uint64_t> hist(32 * 32);
            s = nf_stat_phitheta(h, 32, 32, hist.data());
            if (s == NF_OK) s = nf_format_write_rho("rho.dat", 32, 32, hist.data());
            if (s != NF_OK) { rc = fail(h, s, "stat_phitheta"); goto done; }
            std::printf("file rho.dat created!\n");
        } else if (v.name == "stat_mutangle" || v.name == "stat_contacts") {
            std::vector<uint64_t> hist(32);
            nf_pair_stats ps;
            s = nf_stat_pairs(h, 32, hist.data(), nullptr, 0, &ps);
            if (s != NF_OK) { rc = fail(h, s, v.name.c_str()); goto done; }
            if (v.name == "stat_mutangle") {
                s = nf_format_write_gamma("gamma.dat", 32, hist.data());
                if (s != NF_OK) { rc = fail(h, s, "gamma.dat"); goto done; }
                std::printf("accumulated counts %llu\n", (unsigned long long)ps.angle_pairs);
            } else {
                std::printf(" Total number of contacts per inclusion: %llu / %llu = %f \n",
                            (unsigned long long)ps.contacts_total, (unsigned long long)ps.rods, ps.mean_per_rod);
                std::printf("Maximum number of contacts per inclusion: %u \n", ps.max_per_rod);
            }
        } else if (v.name == "write_ort") {
            s = nf_write_ort_vtk(h, "orient.vtk");
            if (s != NF_OK) { rc = fail(h, s, "write_ort"); goto done; }
        } else if (v.name == "write_lmp") {
            s = nf_write_lmp(h, "output.lmp.data", 4.579);  // simPrms density (src/simPrms.cpp:27)
            if (s != NF_OK) { rc = fail(h, s, "write_lmp"); goto done; }
        } else if (v.name == "reduce") {
            // src/NanoFiller.cpp:71-91: min_cont = 2, then reduced.bin
            const int min_cont = 2;
            std::printf("Eliminating inclusions with less then %d contacts up to %f um:\n", min_cont,
                        p.stat_dist_lim);
            nf_reduce_stats rs;
            s = nf_reduce(h, min_cont, &rs);
            if (s != NF_OK) { rc = fail(h, s, "reduce"); goto done; }
            std::printf("Inclusions remained: %llu of %llu after %d pass(es), %.3f ms\n",
                        (unsigned long long)rs.rods_after, (unsigned long long)rs.rods_before, rs.rounds + 1,
                        rs.ms);
            if (p.wrt_bin) {
                s = nf_write_state_bin(h, "reduced.bin");
                if (s != NF_OK) { rc = fail(h, s, "reduced.bin"); goto done; }
            }
        } else if (v.name == "stat_conduct") {
            nf_contact_stats c;
            s = nf_contacts(h, &c);
            if (s != NF_OK) { rc = fail(h, s, "contacts"); goto done; }
            std::printf("%llu contacts (%llu screened), %llu to the source, %llu to the sink\n",
                        (unsigned long long)c.contacts, (unsigned long long)c.screened,
                        (unsigned long long)c.n_source, (unsigned long long)c.n_sink);
            if (v.internal) {
                nf_internal_stats is;
                s = nf_internal_network(h, &is);
                if (s != NF_OK) { rc = fail(h, s, "internal network"); goto done; }
                s = nf_write_internal_coo(h, ".");
                if (s != NF_OK) { rc = fail(h, s, "internal network files"); goto done; }
                std::printf("%llu nodes (%llu contact ends), %llu rod segments\n", (unsigned long long)is.nodes,
                            (unsigned long long)is.contact_ends, (unsigned long long)is.segments);
            } else {
                s = nf_write_coo(h, ".");
                if (s != NF_OK) { rc = fail(h, s, "coo files"); goto done; }
            }
            nf_solve_stats so;
            s = nf_solve(h, &so);
            if (s != NF_OK && s != NF_ERR_NOT_CONVERGED) { rc = fail(h, s, "solve"); goto done; }
            std::printf("G_eff = %.9e S (%lld of %lld nodes in the network, residual %.3e)\n", so.G_eff,
                        (long long)so.n_active, (long long)so.n_nodes, so.residual);
            if (s == NF_ERR_NOT_CONVERGED) { rc = fail(h, s, "solve"); goto done; }
        }
        // expand only sets the field axis, applied before nf_create.
    }
done:
    nf_destroy(h);
    return rc;
}
