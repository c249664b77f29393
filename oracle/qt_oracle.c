/*
 * qt_oracle.c — TEST INFRASTRUCTURE, NOT THE PRODUCT.  See qt_oracle.h.
 *
 * Plain C11, built with -ffp-contract=off so that every complex product is
 * rounded as (ar*br - ai*bi, ar*bi + ai*br) followed by a separate add, which
 * is what the reference's std::complex<double> loop compiles to on x86-64.
 */
#define _POSIX_C_SOURCE 200809L
#include "qt_oracle.h"

#include <complex.h>
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define QTO_PI 3.14159265358979323846 /* src/Node.h:45 */

/* ------------------------------------------------------------------ */
/* ContractIndices (src/Network.h:876-971)                             */
/* ------------------------------------------------------------------ */

void qto_contract_indices(int rank_a, const double *a, int rank_b, const double *b,
                          int n_free, const int *free_from_a, const int *free_idx,
                          int n_sum, const int *sum_a, const int *sum_b, double *c) {
    int ia[64], ib[64];
    uint64_t n_c = 1ull << (2 * n_free);
    uint64_t n_k = 1ull << (2 * n_sum);
    memset(ia, 0, sizeof ia);
    memset(ib, 0, sizeof ib);
    for (uint64_t cc = 0; cc < n_c; cc++) {
        /* outer digit i of Ccounter <-> toNotSumOn[i]  (Network.h:902-908) */
        for (int i = 0; i < n_free; i++) {
            int d = (int) ((cc >> (2 * i)) & 3u);
            if (free_from_a[i]) ia[free_idx[i]] = d;
            else ib[free_idx[i]] = d;
        }
        double cre = 0.0, cim = 0.0; /* Node(rank) zero-fills (Node.h:113) */
        for (uint64_t k = 0; k < n_k; k++) {
            /* inner digit i of ABcounter <-> toSumOn[K-1-i]  (Network.h:912-916) */
            for (int i = 0; i < n_sum; i++) {
                int d = (int) ((k >> (2 * i)) & 3u);
                ia[sum_a[n_sum - 1 - i]] = d;
                ib[sum_b[n_sum - 1 - i]] = d;
            }
            uint64_t sa = 0, sb = 0;
            for (int j = 0; j < rank_a; j++) sa += (uint64_t) ia[j] << (2 * j);
            for (int j = 0; j < rank_b; j++) sb += (uint64_t) ib[j] << (2 * j);
            double ar = a[2 * sa], ai = a[2 * sa + 1];
            double br = b[2 * sb], bi = b[2 * sb + 1];
            double pre = ar * br - ai * bi;
            double pim = ar * bi + ai * br;
            cre = cre + pre;
            cim = cim + pim;
        }
        c[2 * cc] = cre;
        c[2 * cc + 1] = cim;
    }
}

/* ------------------------------------------------------------------ */
/* Gate tensors (src/Node.h:197-898)                                   */
/* ------------------------------------------------------------------ */

/* flat index of a rank-r tensor entry given its per-wire digits */
static int fidx(int n, const int *d) {
    int s = 0, m = 1;
    for (int i = 0; i < n; i++) { s += d[i] * m; m *= 4; }
    return s;
}

static void set1(double *t, int i0, int i1, double re, double im) {
    int d[2] = {i0, i1};
    int f = fidx(2, d);
    t[2 * f] = re;
    t[2 * f + 1] = im;
}

static void set2(double *t, int i0, int i1, int i2, int i3, double re, double im) {
    int d[4] = {i0, i1, i2, i3};
    int f = fidx(4, d);
    t[2 * f] = re;
    t[2 * f + 1] = im;
}

/* a * conj(b), rounded like std::complex<double> operator* */
static void mul_conj(const double *x, const double *y, double *out) {
    double ar = x[0], ai = x[1], br = y[0], bi = -y[1];
    out[0] = ar * br - ai * bi;
    out[1] = ar * bi + ai * br;
}

/* Superoperator of a 1-qubit U (row-major u[2*row+col]), T[in + 4*out] with
 * in = 2r + c, out = 2r' + c' and T = U[r'][r] * conj(U[c'][c])
 * (the layout of ArbitraryOneQubitNode::ParseMatrixValues, Node.h). */
static void superop1(const double *u, double *t) {
    for (int in = 0; in < 4; in++)
        for (int out = 0; out < 4; out++) {
            int r = in >> 1, c = in & 1, rp = out >> 1, cp = out & 1;
            double v[2];
            mul_conj(&u[2 * (2 * rp + r)], &u[2 * (2 * cp + c)], v);
            set1(t, in, out, v[0], v[1]);
        }
}

/* 2-qubit: wires [in_q1, in_q2, out_q1, out_q2], in_k = 2 r_k + c_k,
 * T = U[2r1'+r2'][2r1+r2] * conj(U[2c1'+c2'][2c1+c2]) (ArbitraryTwoQubitNode). */
static void superop2(const double *u, double *t) {
    for (int i1 = 0; i1 < 4; i1++)
        for (int i2 = 0; i2 < 4; i2++)
            for (int o1 = 0; o1 < 4; o1++)
                for (int o2 = 0; o2 < 4; o2++) {
                    int r1 = i1 >> 1, c1 = i1 & 1, r2 = i2 >> 1, c2 = i2 & 1;
                    int p1 = o1 >> 1, q1 = o1 & 1, p2 = o2 >> 1, q2 = o2 & 1;
                    int row_r = 2 * p1 + p2, col_r = 2 * r1 + r2;
                    int row_c = 2 * q1 + q2, col_c = 2 * c1 + c2;
                    double v[2];
                    mul_conj(&u[2 * (4 * row_r + col_r)], &u[2 * (4 * row_c + col_c)], v);
                    set2(t, i1, i2, o1, o2, v[0], v[1]);
                }
}

/* permutation-like 2-qubit gates with entries +-1 only */
static void superop2_real(const double *ure, double *t) {
    double u[32];
    for (int i = 0; i < 16; i++) { u[2 * i] = ure[i]; u[2 * i + 1] = 0.0; }
    superop2(u, t);
}

int qto_gate_tensor(const char *name, double param, double *out) {
    int rank;
    if (!strcmp(name, "INIT") || !strcmp(name, "T") || !strcmp(name, "MX") || !strcmp(name, "MY") ||
        !strcmp(name, "MZ") || !strcmp(name, "M0") || !strcmp(name, "M1")) rank = 1;
    else if (!strcmp(name, "CNOT") || !strcmp(name, "CZ") || !strcmp(name, "SWAP") ||
             !strcmp(name, "CPHASE") || !strcmp(name, "CRk")) rank = 4;
    else if (!strcmp(name, "Rx") || !strcmp(name, "Ry") || !strcmp(name, "Rz") || !strcmp(name, "PHASE") ||
             !strcmp(name, "H") || !strcmp(name, "X") || !strcmp(name, "Y") || !strcmp(name, "Z")) rank = 2;
    else return -1;
    int n = 1 << (2 * rank);
    memset(out, 0, sizeof(double) * 2 * n);

    if (rank == 1) {
        /* rank-1 nodes are vectors over s = 2r + c (Node.h ZeroStateNode .. ProjectZero) */
        if (!strcmp(name, "INIT") || !strcmp(name, "M0")) out[0] = 1.0;
        else if (!strcmp(name, "M1")) out[6] = 1.0;
        else if (!strcmp(name, "T")) { out[0] = 1.0; out[6] = 1.0; }
        else if (!strcmp(name, "MZ")) { out[0] = 1.0; out[6] = -1.0; }
        else if (!strcmp(name, "MX")) { out[2] = 1.0; out[4] = 1.0; }
        else if (!strcmp(name, "MY")) { out[3] = 1.0; out[5] = -1.0; }
        return rank;
    }

    if (!strcmp(name, "Rx") || !strcmp(name, "Ry")) {
        /* Node.h RxNode / RyNode: the parser narrows the angle with std::stof */
        double th = (double) (float) param;
        double cc = pow(cos(th / 2.0), 2);
        double ss = pow(sin(th / 2.0), 2);
        double sh = sin(th) / 2.0;
        set1(out, 0, 0, cc, 0); set1(out, 1, 1, cc, 0); set1(out, 2, 2, cc, 0); set1(out, 3, 3, cc, 0);
        if (!strcmp(name, "Rx")) {
            set1(out, 0, 3, ss, 0); set1(out, 1, 2, ss, 0); set1(out, 2, 1, ss, 0); set1(out, 3, 0, ss, 0);
            set1(out, 0, 1, 0, sh); set1(out, 1, 0, 0, sh); set1(out, 2, 3, 0, sh); set1(out, 3, 2, 0, sh);
            set1(out, 0, 2, 0, -1.0 * sh); set1(out, 1, 3, 0, -1.0 * sh);
            set1(out, 2, 0, 0, -1.0 * sh); set1(out, 3, 1, 0, -1.0 * sh);
        } else {
            double mss = -1.0 * pow(sin(th / 2), 2);
            double msh = -1.0 * sin(th) / 2.0;
            set1(out, 0, 3, ss, 0); set1(out, 3, 0, ss, 0);
            set1(out, 1, 2, mss, 0); set1(out, 2, 1, mss, 0);
            set1(out, 0, 1, sh, 0); set1(out, 0, 2, sh, 0); set1(out, 1, 3, sh, 0); set1(out, 2, 3, sh, 0);
            set1(out, 1, 0, msh, 0); set1(out, 2, 0, msh, 0); set1(out, 3, 1, msh, 0); set1(out, 3, 2, msh, 0);
        }
        return rank;
    }
    if (!strcmp(name, "Rz") || !strcmp(name, "PHASE")) {
        double th = (double) (float) param;
        set1(out, 0, 0, 1.0, 0); set1(out, 3, 3, 1.0, 0);
        set1(out, 1, 1, cos(th), -1.0 * sin(th));
        set1(out, 2, 2, cos(th), sin(th));
        return rank;
    }
    if (!strcmp(name, "H")) {
        double u[8] = {1, 0, 1, 0, 1, 0, -1, 0};
        /* entries are exactly +-1/2: build from the unnormalised matrix, then halve */
        superop1(u, out);
        for (int i = 0; i < 2 * n; i++) out[i] *= 0.5;
        return rank;
    }
    if (!strcmp(name, "X") || !strcmp(name, "Y") || !strcmp(name, "Z")) {
        double ux[8] = {0, 0, 1, 0, 1, 0, 0, 0};
        double uy[8] = {0, 0, 0, -1, 0, 1, 0, 0};
        double uz[8] = {1, 0, 0, 0, 0, 0, -1, 0};
        superop1(!strcmp(name, "X") ? ux : !strcmp(name, "Y") ? uy : uz, out);
        return rank;
    }
    if (!strcmp(name, "CNOT") || !strcmp(name, "CZ") || !strcmp(name, "SWAP")) {
        double u[16];
        memset(u, 0, sizeof u);
        for (int x = 0; x < 4; x++) {
            int q1 = x >> 1, q2 = x & 1; /* basis index 2*q1 + q2 */
            if (!strcmp(name, "CNOT")) u[4 * (2 * q1 + (q2 ^ q1)) + x] = 1.0;
            else if (!strcmp(name, "SWAP")) u[4 * (2 * q2 + q1) + x] = 1.0;
            else u[4 * x + x] = (q1 && q2) ? -1.0 : 1.0;
        }
        superop2_real(u, out);
        /* +-0 entries of the reference tables are +0 */
        for (int i = 0; i < 2 * n; i++) if (out[i] == 0.0) out[i] = 0.0;
        return rank;
    }
    if (!strcmp(name, "CPHASE") || !strcmp(name, "CRk")) {
        /* controlled phase diag(1,1,1,e^{i phi}) (Node.h CPhaseNode, CRkNode) */
        double er, ei;   /* e^{-i phi}, stored where only the column factor carries the phase */
        double fr, fi;   /* e^{+i phi} */
        if (!strcmp(name, "CPHASE")) {
            er = cos(param); ei = -1.0 * sin(param);
            fr = cos(param); fi = sin(param);
        } else {
            double d = pow(2, param + 1.0);
            double complex zm = cexp(CMPLX(0.0 * 2.0 * QTO_PI / d, -1.0 * 2.0 * QTO_PI / d));
            double complex zp = cexp(CMPLX(0.0 * 2.0 * QTO_PI / d, 1.0 * 2.0 * QTO_PI / d));
            er = creal(zm); ei = cimag(zm);
            fr = creal(zp); fi = cimag(zp);
        }
        for (int i1 = 0; i1 < 4; i1++)
            for (int i2 = 0; i2 < 4; i2++) {
                /* diagonal gate: out == in on both qubits */
                int r1 = i1 >> 1, c1 = i1 & 1, r2 = i2 >> 1, c2 = i2 & 1;
                int rowph = r1 && r2, colph = c1 && c2;
                double vr = 1.0, vi = 0.0;
                if (rowph && !colph) { vr = fr; vi = fi; }
                else if (!rowph && colph) { vr = er; vi = ei; }
                set2(out, i1, i2, i1, i2, vr, vi);
            }
        return rank;
    }
    return -1;
}

/* reads one value the way operator>>(istream&, complex<double>&) accepts it:
 * "(re,im)", "(re)" or "re" */
static int read_complex(const char **p, double *re, double *im) {
    const char *s = *p;
    char *end;
    while (*s == ' ' || *s == '\t' || *s == '\n' || *s == '\r') s++;
    if (!*s) return 0;
    if (*s == '(') {
        s++;
        *re = strtod(s, &end);
        if (end == s) return 0;
        s = end;
        while (*s == ' ') s++;
        if (*s == ',') {
            s++;
            *im = strtod(s, &end);
            if (end == s) return 0;
            s = end;
            while (*s == ' ') s++;
        } else {
            *im = 0.0;
        }
        if (*s != ')') return 0;
        s++;
    } else {
        *re = strtod(s, &end);
        if (end == s) return 0;
        *im = 0.0;
        s = end;
    }
    *p = s;
    return 1;
}

static char *slurp(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *buf = malloc((size_t) n + 1);
    if (fread(buf, 1, (size_t) n, f) != (size_t) n) { fclose(f); free(buf); return NULL; }
    buf[n] = 0;
    fclose(f);
    return buf;
}

int qto_arbitrary_gate(const char *path, int two_qubit, double *out) {
    char *txt = slurp(path);
    if (!txt) return -QTO_INVALID_FILE;
    int nvals = two_qubit ? 16 : 4;
    double u[32];
    const char *p = txt;
    for (int i = 0; i < nvals; i++) {
        if (!read_complex(&p, &u[2 * i], &u[2 * i + 1])) { free(txt); return -QTO_INVALID_FILE_FORMAT; }
    }
    free(txt);
    memset(out, 0, sizeof(double) * 2 * (two_qubit ? 256 : 16));
    if (two_qubit) superop2(u, out);
    else superop1(u, out);
    return two_qubit ? 4 : 2;
}

/* ------------------------------------------------------------------ */
/* Network (src/Network.h)                                             */
/* ------------------------------------------------------------------ */

typedef struct {
    int node_a, node_b;   /* -1 = null endpoint */
    int qubit;
    int contracted;
    int lg_id;
} owire;

typedef struct {
    int rank;
    int nw, capw;
    int *wires;
    double *vals;         /* 2 * 4^rank doubles, NULL once cleared */
    int contracted;
    int created_from[2];
} onode;

struct qto_net {
    int n_qubits;
    onode *nodes; int n_nodes, cap_nodes;
    owire *wires; int n_wires, cap_wires;
    int *uncon; int n_uncon, cap_uncon;
    int *parsing_wires;
    double final_re, final_im;
    int done;
    int64_t flops;
    char def1_names[64][64], def1_paths[64][512]; int n_def1;
    char def2_names[64][64], def2_paths[64][512]; int n_def2;
    const char *gate_dir;
};

static int new_node(qto_net *net, int rank) {
    if (net->n_nodes == net->cap_nodes) {
        net->cap_nodes = net->cap_nodes ? 2 * net->cap_nodes : 64;
        net->nodes = realloc(net->nodes, sizeof(onode) * (size_t) net->cap_nodes);
    }
    onode *n = &net->nodes[net->n_nodes];
    memset(n, 0, sizeof *n);
    n->rank = rank;
    n->vals = calloc((size_t) 2 << (2 * rank), sizeof(double));
    return net->n_nodes++;
}

static int new_wire(qto_net *net, int a, int b, int qubit) {
    if (net->n_wires == net->cap_wires) {
        net->cap_wires = net->cap_wires ? 2 * net->cap_wires : 64;
        net->wires = realloc(net->wires, sizeof(owire) * (size_t) net->cap_wires);
    }
    owire *w = &net->wires[net->n_wires];
    w->node_a = a; w->node_b = b; w->qubit = qubit; w->contracted = 0; w->lg_id = -1;
    return net->n_wires++;
}

static void node_add_wire(qto_net *net, int node, int wire) {
    onode *n = &net->nodes[node];
    if (n->nw == n->capw) {
        n->capw = n->capw ? 2 * n->capw : 4;
        n->wires = realloc(n->wires, sizeof(int) * (size_t) n->capw);
    }
    n->wires[n->nw++] = wire;
}

static void uncon_push(qto_net *net, int node) {
    if (net->n_uncon == net->cap_uncon) {
        net->cap_uncon = net->cap_uncon ? 2 * net->cap_uncon : 64;
        net->uncon = realloc(net->uncon, sizeof(int) * (size_t) net->cap_uncon);
    }
    net->uncon[net->n_uncon++] = node;
}

void qto_net_free(qto_net *net) {
    if (!net) return;
    for (int i = 0; i < net->n_nodes; i++) { free(net->nodes[i].wires); free(net->nodes[i].vals); }
    free(net->nodes); free(net->wires); free(net->uncon); free(net->parsing_wires);
    free(net);
}

/* std::stoi / std::stof-like: must consume at least one character */
static int parse_int(const char *s, int *out) {
    char *end;
    errno = 0;
    long v = strtol(s, &end, 10);
    if (end == s || errno) return 0;
    *out = (int) v;
    return 1;
}

static int parse_float(const char *s, float *out) {
    char *end;
    errno = 0;
    float v = strtof(s, &end);
    if (end == s || errno == ERANGE) return 0;
    *out = v;
    return 1;
}

static int parse_double(const char *s, double *out) {
    char *end;
    errno = 0;
    double v = strtod(s, &end);
    if (end == s || errno == ERANGE) return 0;
    *out = v;
    return 1;
}

/* attach a gate node to the hanging wires of its qubits (Network.h:356-378, 522-536) */
static void attach(qto_net *net, int node, const int *qubits, int nq) {
    for (int i = 0; i < nq; i++) {
        int w = net->parsing_wires[qubits[i]];
        node_add_wire(net, node, w);
        net->wires[w].node_b = node;
    }
    for (int i = 0; i < nq; i++) {
        int w = new_wire(net, node, -1, qubits[i]);
        net->parsing_wires[qubits[i]] = w;
        node_add_wire(net, node, w);
    }
}

/* tokenizer of Network.h:976-992: split on single spaces, keep empty tokens,
 * drop only an empty final piece; lines starting with '#' are comments */
static int tokenize(char *line, char **tok, int cap) {
    size_t len = strlen(line);
    if (len == 0 || line[0] == '#') return 0;
    int n = 0;
    char *s = line;
    for (;;) {
        char *sp = strchr(s, ' ');
        if (!sp) {
            if (*s && n < cap) tok[n++] = s;
            break;
        }
        *sp = 0;
        if (n < cap) tok[n++] = s;
        s = sp + 1;
    }
    return n;
}

static const char *lookup(char names[][64], char paths[][512], int n, const char *key) {
    for (int i = 0; i < n; i++) if (!strcmp(names[i], key)) return paths[i];
    return NULL;
}

static int parse_line(qto_net *net, char *line) {
    char *tok[64];
    int nt = tokenize(line, tok, 64);
    if (nt == 0) return QTO_OK;
    int nq = net->n_qubits;
    const char *g = tok[0];
    int node = -1;
    int q[2];
    double t[512];
    const char *arb1 = NULL, *arb2 = NULL;

    if (!strcmp(g, "Rx") || !strcmp(g, "RX") || !strcmp(g, "Ry") || !strcmp(g, "RY") ||
        !strcmp(g, "Rz") || !strcmp(g, "RZ") || !strcmp(g, "PHASE")) {
        float th;
        if (nt < 3 || !parse_float(tok[1], &th) || !parse_int(tok[2], &q[0])) return QTO_INVALID_FILE_FORMAT;
        if (q[0] > nq - 1 || q[0] < 0) return QTO_INVALID_FILE_FORMAT;
        const char *kind = (g[1] == 'x' || g[1] == 'X') ? "Rx" : (g[1] == 'y' || g[1] == 'Y') ? "Ry"
                         : (!strcmp(g, "PHASE")) ? "PHASE" : "Rz";
        node = new_node(net, 2);
        qto_gate_tensor(kind, (double) th, net->nodes[node].vals);
        attach(net, node, q, 1);
    } else if (!strcmp(g, "H") || !strcmp(g, "X") || !strcmp(g, "Y") || !strcmp(g, "Z")) {
        if (nt < 2 || !parse_int(tok[1], &q[0])) return QTO_INVALID_FILE_FORMAT;
        if (q[0] > nq - 1 || q[0] < 0) return QTO_INVALID_FILE_FORMAT;
        node = new_node(net, 2);
        qto_gate_tensor(g, 0.0, net->nodes[node].vals);
        attach(net, node, q, 1);
    } else if (!strcmp(g, "CNOT") || !strcmp(g, "SWAP") || !strcmp(g, "CRk") || !strcmp(g, "CZ")) {
        if (nt < 3 || !parse_int(tok[1], &q[0]) || !parse_int(tok[2], &q[1])) return QTO_INVALID_FILE_FORMAT;
        if (q[0] > nq - 1 || q[1] > nq - 1 || q[0] == q[1] || q[0] < 0 || q[1] < 0) return QTO_INVALID_FILE_FORMAT;
        node = new_node(net, 4);
        /* CRk's phase uses the control qubit index (Network.h:571) */
        qto_gate_tensor(g, (double) q[0], net->nodes[node].vals);
        attach(net, node, q, 2);
    } else if (!strcmp(g, "CPHASE")) {
        double th;
        if (nt < 4 || !parse_double(tok[1], &th) || !parse_int(tok[2], &q[0]) || !parse_int(tok[3], &q[1]))
            return QTO_INVALID_FILE_FORMAT;
        if (q[0] > nq - 1 || q[1] > nq - 1 || q[0] == q[1] || q[0] < 0 || q[1] < 0) return QTO_INVALID_FILE_FORMAT;
        node = new_node(net, 4);
        qto_gate_tensor("CPHASE", th, net->nodes[node].vals);
        attach(net, node, q, 2);
    } else if (!strcmp(g, "def1") || !strcmp(g, "def2")) {
        if (nt < 3) return QTO_INVALID_FILE_FORMAT;
        int two = g[3] == '2';
        char (*names)[64] = two ? net->def2_names : net->def1_names;
        char (*paths)[512] = two ? net->def2_paths : net->def1_paths;
        int *cnt = two ? &net->n_def2 : &net->n_def1;
        /* unordered_map::insert keeps the first definition */
        if (!lookup(names, paths, *cnt, tok[1]) && *cnt < 64) {
            snprintf(names[*cnt], 64, "%s", tok[1]);
            snprintf(paths[*cnt], 512, "%s", tok[2]);
            (*cnt)++;
        }
        return QTO_OK;
    } else if ((arb1 = lookup(net->def1_names, net->def1_paths, net->n_def1, g)) != NULL) {
        if (nt < 2 || !parse_int(tok[1], &q[0])) return QTO_INVALID_FILE_FORMAT;
        char path[1024];
        if (net->gate_dir && arb1[0] != '/') snprintf(path, sizeof path, "%s/%s", net->gate_dir, arb1);
        else snprintf(path, sizeof path, "%s", arb1);
        int r = qto_arbitrary_gate(path, 0, t);
        if (r < 0) return -r;
        if (q[0] > nq - 1 || q[0] < 0) return QTO_INVALID_FILE_FORMAT;
        node = new_node(net, 2);
        memcpy(net->nodes[node].vals, t, sizeof(double) * 32);
        attach(net, node, q, 1);
    } else if ((arb2 = lookup(net->def2_names, net->def2_paths, net->n_def2, g)) != NULL) {
        char path[1024];
        if (net->gate_dir && arb2[0] != '/') snprintf(path, sizeof path, "%s/%s", net->gate_dir, arb2);
        else snprintf(path, sizeof path, "%s", arb2);
        int r = qto_arbitrary_gate(path, 1, t);
        if (r < 0) return -r;
        if (nt < 3 || !parse_int(tok[1], &q[0]) || !parse_int(tok[2], &q[1])) return QTO_INVALID_FILE_FORMAT;
        if (q[0] > nq - 1 || q[1] > nq - 1 || q[0] == q[1] || q[0] < 0 || q[1] < 0) return QTO_INVALID_FILE_FORMAT;
        node = new_node(net, 4);
        memcpy(net->nodes[node].vals, t, sizeof(double) * 512);
        attach(net, node, q, 2);
    } else {
        return QTO_INVALID_FILE_FORMAT;
    }
    return QTO_OK;
}

qto_net *qto_net_parse(const char *qasm_text, const char *measure_text, const char *gate_dir, int *err) {
    *err = QTO_OK;
    if (!qasm_text) { *err = QTO_INVALID_FILE; return NULL; }
    qto_net *net = calloc(1, sizeof(qto_net));
    net->gate_dir = gate_dir;
    char *txt = strdup(qasm_text);
    /* std::getline splits on '\n' */
    char *line = txt;
    char *nl = strchr(line, '\n');
    if (nl) *nl = 0;
    int nq;
    if (!parse_int(line, &nq) || nq < 0) { free(txt); qto_net_free(net); *err = QTO_INVALID_FILE_FORMAT; return NULL; }
    net->n_qubits = nq;
    net->parsing_wires = calloc((size_t) (nq > 0 ? nq : 1), sizeof(int));
    /* initial |0><0| states, ids 0..n-1 (Network.h:177-194) */
    for (int i = 0; i < nq; i++) {
        int nd = new_node(net, 1);
        qto_gate_tensor("INIT", 0, net->nodes[nd].vals);
        int w = new_wire(net, nd, -1, i);
        node_add_wire(net, nd, w);
        net->parsing_wires[i] = w;
    }
    while (nl) {
        line = nl + 1;
        nl = strchr(line, '\n');
        if (nl) *nl = 0;
        int rc = parse_line(net, line);
        if (rc != QTO_OK) { free(txt); qto_net_free(net); *err = rc; return NULL; }
    }
    free(txt);
    /* measurements: one non-space char per qubit, missing -> trace (Network.h:285-299) */
    const char *m = measure_text ? measure_text : "";
    for (int i = 0; i < nq; i++) {
        while (*m == ' ' || *m == '\t' || *m == '\n' || *m == '\r' || *m == '\v' || *m == '\f') m++;
        char ch = 'T';
        if (*m) ch = *m++;
        const char *kind = ch == 'X' ? "MX" : ch == 'Y' ? "MY" : ch == 'Z' ? "MZ" : ch == '0' ? "M0" : ch == '1' ? "M1" : "T";
        int nd = new_node(net, 1);
        qto_gate_tensor(kind, 0, net->nodes[nd].vals);
        int w = net->parsing_wires[i];
        net->wires[w].node_b = nd;
        node_add_wire(net, nd, w);
    }
    for (int i = 0; i < net->n_nodes; i++) uncon_push(net, i);
    return net;
}

int qto_net_num_qubits(const qto_net *net) { return net->n_qubits; }
int qto_net_num_nodes(const qto_net *net) { return net->n_nodes; }
int qto_net_node_rank(const qto_net *net, int id) { return net->nodes[id].rank; }

int qto_net_node_values(const qto_net *net, int id, double *out, int64_t cap) {
    const onode *n = &net->nodes[id];
    if (!n->vals) return 0;
    int64_t cnt = (int64_t) 2 << (2 * n->rank);
    if (cnt > cap) return -1;
    memcpy(out, n->vals, sizeof(double) * (size_t) cnt);
    return 1;
}

static int wire_touches(const owire *w, int node) { return w->node_b == node || w->node_a == node; }

int qto_net_contract(qto_net *net, int id_a, int id_b, int threshold) {
    onode *A = &net->nodes[id_a];
    onode *B = &net->nodes[id_b];
    if (A->contracted || B->contracted) return -1;
    int ia[64], ib[64], nsa = 0, nsb = 0;
    int cfa[128], cfi[128], nc = 0;
    int conn[64], nconn = 0, rem[128], nrem = 0;
    for (int i = 0; i < A->nw; i++) {
        const owire *w = &net->wires[A->wires[i]];
        if (wire_touches(w, id_b)) { ia[nsa++] = i; conn[nconn++] = A->wires[i]; }
        else { cfa[nc] = 1; cfi[nc] = i; nc++; rem[nrem++] = A->wires[i]; }
    }
    for (int j = 0; j < nconn; j++)
        for (int k = 0; k < B->nw; k++)
            if (conn[j] == B->wires[k]) ib[nsb++] = k;
    for (int j = 0; j < B->nw; j++) {
        const owire *w = &net->wires[B->wires[j]];
        if (!wire_touches(w, id_a)) { cfa[nc] = 0; cfi[nc] = j; nc++; rem[nrem++] = B->wires[j]; }
    }
    int mx = A->rank > B->rank ? A->rank : B->rank;
    if ((nsa == 0 && nc > 0) || nrem > mx + threshold) return -1;
    if (!A->vals || !B->vals) return -1;
    int idc = new_node(net, nc);
    A = &net->nodes[id_a];   /* realloc may have moved the array */
    B = &net->nodes[id_b];
    onode *C = &net->nodes[idc];
    for (int i = 0; i < nrem; i++) {
        owire *w = &net->wires[rem[i]];
        node_add_wire(net, idc, rem[i]);
        C = &net->nodes[idc];
        if (w->node_a == id_a || w->node_a == id_b) w->node_a = idc;
        else if (w->node_b == id_a || w->node_b == id_b) w->node_b = idc;
    }
    A->contracted = 1;
    B->contracted = 1;
    for (int i = 0; i < nconn; i++) net->wires[conn[i]].contracted = 1;
    net->flops += (int64_t) 1 << (2 * (nc + nsa));
    qto_contract_indices(A->rank, A->vals, B->rank, B->vals, nc, cfa, cfi, nsa, ia, ib, C->vals);
    if (nc == 0) {
        if ((fabs(net->final_re) <= 1.0e-30 && fabs(net->final_im) <= 1.0e-30) || (A->rank == 0 && B->rank == 0)) {
            net->final_re = C->vals[0];
            net->final_im = C->vals[1];
        }
        if (net->n_uncon == 2) net->done = 1;
    }
    /* mAllNodes gets C, or a zero-valued rank-0 placeholder once done (Network.h:841-863) */
    int pos_a = -1;
    for (int i = 0; i < net->n_uncon; i++) if (net->uncon[i] == id_a) { pos_a = i; break; }
    if (pos_a >= 0) {
        memmove(&net->uncon[pos_a], &net->uncon[pos_a + 1], sizeof(int) * (size_t) (net->n_uncon - pos_a - 1));
        net->n_uncon--;
    }
    int result = idc;
    if (net->done) {
        /* the placeholder takes the next id; C itself only lives in the uncontracted list */
        int ph = new_node(net, 0);
        net->nodes[ph].created_from[0] = id_a;
        net->nodes[ph].created_from[1] = id_b;
        /* swap so that ids stay reference-compatible: placeholder at idc, C after it */
        onode tmp = net->nodes[idc];
        net->nodes[idc] = net->nodes[ph];
        net->nodes[ph] = tmp;
        /* the C node now sits at index ph; it is not part of mAllNodes' id space */
        for (int i = 0; i < net->n_uncon; i++) if (net->uncon[i] == id_b) { net->uncon[i] = ph; break; }
        for (int i = 0; i < net->nodes[ph].nw; i++) {
            owire *w = &net->wires[net->nodes[ph].wires[i]];
            if (w->node_a == idc) w->node_a = ph;
            else if (w->node_b == idc) w->node_b = ph;
        }
        result = -2;
    } else {
        net->nodes[idc].created_from[0] = id_a;
        net->nodes[idc].created_from[1] = id_b;
        for (int i = 0; i < net->n_uncon; i++) if (net->uncon[i] == id_b) { net->uncon[i] = idc; break; }
    }
    onode *An = &net->nodes[id_a], *Bn = &net->nodes[id_b];
    free(An->vals); An->vals = NULL;
    free(Bn->vals); Bn->vals = NULL;
    return result;
}

int qto_net_replay(qto_net *net, const int *pairs, int n_pairs) {
    for (int i = 0; i < n_pairs; i++) {
        int a = pairs[2 * i], b = pairs[2 * i + 1];
        if (a < 0 || b < 0 || a >= net->n_nodes || b >= net->n_nodes) return QTO_INVALID_FUNCTION_INPUT;
        qto_net_contract(net, a, b, 100);
    }
    return net->done ? QTO_OK : QTO_CONTRACTION_FAILURE;
}

static int lg_number(qto_net *net, int *wire_of_id) {
    /* LineGraph.h:92-130: ids in first-seen order over the uncontracted nodes' wire lists */
    int n = 0;
    for (int i = 0; i < net->n_wires; i++) net->wires[i].lg_id = -1;
    for (int u = 0; u < net->n_uncon; u++) {
        onode *nd = &net->nodes[net->uncon[u]];
        for (int k = 0; k < nd->nw; k++) {
            owire *w = &net->wires[nd->wires[k]];
            if (w->lg_id < 0) {
                w->lg_id = n;
                if (wire_of_id) wire_of_id[n] = nd->wires[k];
                n++;
            }
        }
    }
    return n;
}

int qto_net_lg_wire_ids(qto_net *net, int *node_ids, int *ranks, int *wire_ids, int cap) {
    int total = lg_number(net, NULL);
    int pos = 0;
    for (int u = 0; u < net->n_uncon; u++) {
        onode *nd = &net->nodes[net->uncon[u]];
        node_ids[u] = net->uncon[u];
        ranks[u] = nd->nw;
        for (int k = 0; k < nd->nw && pos < cap; k++) wire_ids[pos++] = net->wires[nd->wires[k]].lg_id;
    }
    return total;
}

int qto_net_lg_contract(qto_net *net, const int *order, int n) {
    int *wire_of_id = malloc(sizeof(int) * (size_t) (net->n_wires + 1));
    int nw = lg_number(net, wire_of_id);
    for (int i = 0; i < n && i < nw; i++) {
        int id = order[i] - 1;
        if (id < 0 || id >= nw) { free(wire_of_id); return QTO_INVALID_FUNCTION_INPUT; }
        owire *w = &net->wires[wire_of_id[id]];
        if (!w->contracted) {
            if (w->node_a < 0 || w->node_b < 0) continue;
            qto_net_contract(net, w->node_a, w->node_b, 100);
        }
    }
    free(wire_of_id);
    if (net->n_uncon != 1) return QTO_CONTRACTION_FAILURE;
    if (net->nodes[net->uncon[0]].rank != 0) return QTO_CONTRACTION_FAILURE;
    return QTO_OK;
}

int qto_net_done(const qto_net *net) { return net->done; }

void qto_net_final_value(const qto_net *net, double *v) { v[0] = net->final_re; v[1] = net->final_im; }

int64_t qto_net_flops(const qto_net *net) { return net->flops; }

int qto_net_created_from(const qto_net *net, int *pairs, int cap) {
    int n = 0;
    for (int i = 0; i < net->n_nodes; i++) {
        const onode *nd = &net->nodes[i];
        if (!(nd->created_from[0] == 0 && nd->created_from[1] == 0)) {
            if (n < cap) { pairs[2 * n] = nd->created_from[0]; pairs[2 * n + 1] = nd->created_from[1]; }
            n++;
        }
    }
    return n;
}

int qto_net_remaining_value(const qto_net *net, double *v) {
    if (net->n_uncon != 1) return QTO_CONTRACTION_FAILURE;
    const onode *nd = &net->nodes[net->uncon[0]];
    if (!nd->vals || nd->rank != 0) return QTO_CONTRACTION_FAILURE;
    v[0] = nd->vals[0];
    v[1] = nd->vals[1];
    return QTO_OK;
}
