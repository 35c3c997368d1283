// host_config.cpp -- ebb-solve JSON config (source/config.d:112-313) and the
// manufactured-solution fields used by Dirichlet boundaries and source terms.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "host.hpp"

namespace ebb {
namespace {

// ---- minimal JSON value + recursive-descent parser -------------------------
struct JVal {
    enum Kind { NUL, TRUE_, FALSE_, INT, FLOAT, STR, ARR, OBJ } kind = NUL;
    long long i = 0;
    double f = 0;
    std::string s;
    std::vector<JVal> a;
    std::vector<std::pair<std::string, JVal>> o;
    const JVal *get(const char *k) const
    {
        if (kind != OBJ) return nullptr;
        for (auto &kv : o)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
    bool is_num() const { return kind == INT || kind == FLOAT; }
    double num() const { return kind == INT ? (double)i : f; }
};

struct Parser {
    const char *p;
    std::string err;
    void ws()
    {
        while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') p++;
    }
    bool str(std::string &out)
    {
        if (*p != '"') return false;
        p++;
        while (*p && *p != '"') {
            if (*p == '\\') {
                p++;
                switch (*p) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': {
                    unsigned v = (unsigned)std::strtoul(std::string(p + 1, 4).c_str(), nullptr, 16);
                    out += (char)(v & 0x7f);
                    p += 4;
                    break;
                }
                default: out += *p;
                }
                if (*p) p++;
            } else {
                out += *p++;
            }
        }
        if (*p != '"') return false;
        p++;
        return true;
    }
    bool value(JVal &v)
    {
        ws();
        if (*p == '{') {
            v.kind = JVal::OBJ;
            p++;
            ws();
            if (*p == '}') {
                p++;
                return true;
            }
            for (;;) {
                ws();
                std::string k;
                if (!str(k)) return false;
                ws();
                if (*p != ':') return false;
                p++;
                JVal c;
                if (!value(c)) return false;
                v.o.emplace_back(k, std::move(c));
                ws();
                if (*p == ',') {
                    p++;
                    continue;
                }
                if (*p == '}') {
                    p++;
                    return true;
                }
                return false;
            }
        }
        if (*p == '[') {
            v.kind = JVal::ARR;
            p++;
            ws();
            if (*p == ']') {
                p++;
                return true;
            }
            for (;;) {
                JVal c;
                if (!value(c)) return false;
                v.a.push_back(std::move(c));
                ws();
                if (*p == ',') {
                    p++;
                    continue;
                }
                if (*p == ']') {
                    p++;
                    return true;
                }
                return false;
            }
        }
        if (*p == '"') {
            v.kind = JVal::STR;
            return str(v.s);
        }
        if (!std::strncmp(p, "true", 4)) {
            v.kind = JVal::TRUE_;
            p += 4;
            return true;
        }
        if (!std::strncmp(p, "false", 5)) {
            v.kind = JVal::FALSE_;
            p += 5;
            return true;
        }
        if (!std::strncmp(p, "null", 4)) {
            v.kind = JVal::NUL;
            p += 4;
            return true;
        }
        // number: INT unless it has '.', 'e' or 'E' (std.json semantics)
        const char *s = p;
        if (*p == '-' || *p == '+') p++;
        bool isf = false;
        while ((*p >= '0' && *p <= '9') || *p == '.' || *p == 'e' || *p == 'E' || *p == '-' || *p == '+') {
            if (*p == '.' || *p == 'e' || *p == 'E') isf = true;
            p++;
        }
        if (p == s) return false;
        std::string tok(s, p - s);
        char *e;
        if (isf) {
            v.kind = JVal::FLOAT;
            v.f = std::strtod(tok.c_str(), &e);
        } else {
            v.kind = JVal::INT;
            v.i = std::strtoll(tok.c_str(), &e, 10);
        }
        return *e == 0;
    }
};

void copy_str(char *dst, size_t n, const std::string &s)
{
    size_t k = std::min(n - 1, s.size());
    std::memcpy(dst, s.data(), k);
    dst[k] = 0;
}

}  // namespace

bool parse_config_json(const char *text, ebb_config *c, std::string &err)
{
    ebb_config_defaults(c);
    Parser P{text, ""};
    JVal root;
    if (!P.value(root) || root.kind != JVal::OBJ) {
        err = "config is not a JSON object";
        return false;
    }
    auto need = [&](const char *k) -> const JVal * {
        const JVal *v = root.get(k);
        if (!v) err = std::string("missing required key \"") + k + "\"";
        return v;
    };
    const JVal *v;
    if (!(v = need("mesh")) || v->kind != JVal::STR) return err.empty() ? (err = "mesh must be a string", false) : false;
    copy_str(c->mesh_file, EBB_PATH_LEN, v->s);
    if (!(v = need("flux")) || v->kind != JVal::STR) return err.empty() ? (err = "flux must be a string", false) : false;
    if (v->s == "rusanovFlux")
        c->flux = EBB_FLUX_RUSANOV;
    else if (v->s == "roeFlux")
        c->flux = EBB_FLUX_ROE;
    else {
        err = "unknown flux " + v->s;
        return false;
    }
    // "dt": .floating (config.d:119) -- an integer literal is an error in the reference
    if (!(v = need("dt")) || v->kind != JVal::FLOAT) return err.empty() ? (err = "dt must be a floating-point number", false) : false;
    c->dt = v->f;
    if (!(v = need("tEnd")) || !v->is_num()) return err.empty() ? (err = "tEnd must be a number", false) : false;
    c->t_end = v->num();
    if (!(v = need("saveIter")) || v->kind != JVal::INT) return err.empty() ? (err = "saveIter must be an integer", false) : false;
    c->save_iter = v->i;
    if (!(v = need("plotIter")) || v->kind != JVal::INT) return err.empty() ? (err = "plotIter must be an integer", false) : false;
    c->plot_iter = v->i;
    if (!(v = need("forceBoundary"))) return false;
    c->n_force = 0;
    if (v->kind == JVal::ARR) {
        for (auto &x : v->a) {
            if (x.kind != JVal::STR || c->n_force >= EBB_MAX_FORCE_TAGS) {
                err = "forceBoundary entries must be strings";
                return false;
            }
            copy_str(c->force_boundary[c->n_force++], EBB_TAG_LEN, x.s);
        }
    } else if (v->kind == JVal::STR) {
        copy_str(c->force_boundary[c->n_force++], EBB_TAG_LEN, v->s);
    } else {
        err = "forceBoundary must be a string or an array";
        return false;
    }
    auto flag = [&](const char *k, int32_t def) -> int32_t {
        const JVal *x = root.get(k);
        return x ? (x->kind == JVal::TRUE_) : def;
    };
    if ((v = root.get("CFL"))) {
        if (!v->is_num()) {
            err = "CFL must be a number";
            return false;
        }
        c->cfl = v->num();
    } else {
        c->cfl = 0.5;
    }
    c->dynamic_dt = flag("dynamicDt", 1);
    if ((v = root.get("integrator"))) {
        if (v->kind != JVal::STR) {
            err = "integrator must be a string";
            return false;
        }
        if (v->s == "Euler")
            c->integrator = EBB_INT_EULER;
        else if (v->s == "RK2")
            c->integrator = EBB_INT_RK2;
        else if (v->s == "RK2_TVD")
            c->integrator = EBB_INT_RK2_TVD;
        else if (v->s == "RK4")
            c->integrator = EBB_INT_RK4;
        else {
            err = "unknown integrator " + v->s;
            return false;
        }
    } else {
        c->integrator = EBB_INT_EULER;
    }
    c->limited = flag("limited", 1);
    c->local_timestep = flag("localTimestep", 0);
    if ((v = root.get("lpThresh"))) {
        if (!v->is_num()) {
            err = "lpThresh must be a number";
            return false;
        }
        c->lp_thresh = v->num();
    } else {
        c->lp_thresh = -1;
    }
    if ((v = root.get("order")) && v->kind == JVal::INT)
        c->order = (v->i == 1 || v->i == 2) ? v->i : 2;
    else
        c->order = 2;
    c->multistage_limiting = flag("multistageLimiting", 1);
    c->cfl_adjust = flag("cflAdjust", 1);
    c->viscosity = flag("viscosity", 0);
    c->pr = 0.7;
    c->r_gas = 8.3145;
    c->gamma = 1.4;
    c->re = 1000;
    c->l_ref = 1;
    if ((v = root.get("physicalConfig")) && v->kind == JVal::OBJ) {
        const JVal *a = v->get("Pr"), *b = v->get("R"), *g = v->get("gamma"), *r = v->get("Re"), *l = v->get("L");
        if (a && b && g && r && l && a->is_num() && b->is_num() && g->is_num() && r->is_num() && l->is_num()) {
            c->pr = a->num();
            c->r_gas = b->num();
            c->gamma = g->num();
            c->re = r->num();
            c->l_ref = l->num();
        }
    }
    if (!(v = need("initialConditions")) || v->kind != JVal::ARR || v->a.size() < 4)
        return err.empty() ? (err = "initialConditions must hold 4 numbers", false) : false;
    for (int k = 0; k < 4; k++) {
        if (!v->a[k].is_num()) {
            err = "initialConditions must hold numbers";
            return false;
        }
        c->ic[k] = v->a[k].num();
    }
    if (!(v = need("boudaryConditions")) || v->kind != JVal::ARR)
        return err.empty() ? (err = "boudaryConditions must be an array", false) : false;
    if (v->a.size() > EBB_MAX_BC) {
        err = "too many boundary conditions";
        return false;
    }
    c->n_boundaries = (int32_t)v->a.size();
    for (size_t i = 0; i < v->a.size(); i++) {
        const JVal &b = v->a[i];
        const JVal *t = b.get("tag"), *ty = b.get("type"), *q = b.get("q");
        if (!t || t->kind != JVal::STR || !ty || ty->kind != JVal::STR || !q || q->kind != JVal::ARR) {
            err = "boundary condition needs tag, type and q";
            return false;
        }
        ebb_boundary &B = c->boundaries[i];
        copy_str(B.tag, EBB_TAG_LEN, t->s);
        const std::string &s = ty->s;
        // unknown names leave the enum at its default FullState (config.d:273-301)
        B.type = s == "inviscidWall" ? EBB_BC_INVISCID_WALL
                 : s == "viscidWall" ? EBB_BC_VISCOUS_WALL
                 : s == "constP"     ? EBB_BC_CONST_PRESSURE
                 : s == "symmetry"   ? EBB_BC_SYMMETRY
                 : s == "tpInflow"   ? EBB_BC_TEMP_PRES_INFLOW
                 : s == "dirichlet"  ? EBB_BC_DIRICHLET
                                     : EBB_BC_FULL_STATE;
        if (q->a.size() > 8) {
            err = "boundary q has too many entries";
            return false;
        }
        B.n_data = (int32_t)q->a.size();
        for (size_t k = 0; k < q->a.size(); k++) {
            if (!q->a[k].is_num()) {
                err = "boundary q must hold numbers";
                return false;
            }
            B.data[k] = q->a[k].num();
        }
    }
    return true;
}

// ---- manufactured solutions -------------------------------------------------
namespace {
constexpr double AR = 0.9, BR = 0.04, CR = -2, DR = 1;
constexpr double AU = 0.1, BU = 0.02, CU = 1, DU = 1;
constexpr double AV = 0.05, BV = -0.1, CV = 0.7, DV = 1.3;
constexpr double AP = 1, BP = 0.05, CP = 2, DP = -1;
constexpr double G = 1.4;

// manufacturedsolution.d:47-156
double rho(double x, double y) { return AR + BR * std::sin(CR * x + DR * y); }
double drdx(double x, double y) { return BR * CR * std::cos(CR * x + DR * y); }
double d2rdx2(double x, double y) { return -BR * (CR * CR) * std::sin(CR * x + DR * y); }
double drdy(double x, double y) { return BR * DR * std::cos(CR * x + DR * y); }
double d2rdy2(double x, double y) { return -BR * (DR * DR) * std::sin(CR * x + DR * y); }
double uu(double x, double y) { return AU + BU * std::cos(CU * x + DU * y); }
double dudx(double x, double y) { return -BU * CU * std::sin(CU * x + DU * y); }
double d2udxy(double x, double y) { return -BU * CU * DU * std::cos(CU * x + DU * y); }
double d2udx2(double x, double y) { return -BU * (CU * CU) * std::cos(CU * x + DU * y); }
double dudy(double x, double y) { return -BU * DU * std::sin(CU * x + DU * y); }
double d2udy2(double x, double y) { return -BU * (DU * DU) * std::cos(CU * x + DU * y); }
double vv(double x, double y) { return AV + BV * std::cos(CV * x + DV * y); }
double dvdx(double x, double y) { return -BV * CV * std::sin(CV * x + DV * y); }
double dvdy(double x, double y) { return -BV * DV * std::sin(CV * x + DV * y); }
double d2vdx2(double x, double y) { return -BV * (CV * CV) * std::cos(CV * x + DV * y); }
double d2vdy2(double x, double y) { return -BV * (DV * DV) * std::cos(CV * x + DV * y); }
double d2vdxy(double x, double y) { return -BV * CV * DV * std::cos(CV * x + DV * y); }
double pp(double x, double y) { return AP + BP * std::sin(CP * x + DP * y); }
double dpdx(double x, double y) { return BP * CP * std::cos(CP * x + DP * y); }
double d2pdx2(double x, double y) { return -BP * (CP * CP) * std::sin(CP * x + DP * y); }
double dpdy(double x, double y) { return BP * DP * std::cos(CP * x + DP * y); }
double d2pdy2(double x, double y) { return -BP * (DP * DP) * std::sin(CP * x + DP * y); }

double pressure(const double q[4])
{
    double a = q[1] / q[0], b = q[2] / q[0];
    return (G - 1) * (q[3] - 0.5 * q[0] * (a * a + b * b));
}

constexpr double TWO_PI = 6.283185307179586;
void sine_prims(double x, double y, double w[4], double wx[4], double wy[4])
{
    double sx = std::sin(TWO_PI * x), cx = std::cos(TWO_PI * x), sy = std::sin(TWO_PI * y), cy = std::cos(TWO_PI * y);
    double s1 = std::sin(TWO_PI * x + 1.0), c1 = std::cos(TWO_PI * x + 1.0);
    w[0] = 1.0 + 0.1 * sx * cy;
    w[1] = 0.5 + 0.05 * cx * sy;
    w[2] = 0.3 + 0.05 * s1;
    w[3] = 1.0 / 1.4 + 0.1 * cy;
    wx[0] = 0.1 * TWO_PI * cx * cy;
    wy[0] = -0.1 * TWO_PI * sx * sy;
    wx[1] = -0.05 * TWO_PI * sx * sy;
    wy[1] = 0.05 * TWO_PI * cx * cy;
    wx[2] = 0.05 * TWO_PI * c1;
    wy[2] = 0.0;
    wx[3] = 0.0;
    wy[3] = -0.1 * TWO_PI * sy;
}
}  // namespace

void mms_solution(int kind, double x, double y, double q[4])
{
    if (kind == EBB_MMS_SINE) {
        double w[4], wx[4], wy[4];
        sine_prims(x, y, w, wx, wy);
        double r = 1.0 + 0.1 * std::sin(TWO_PI * x) * std::cos(TWO_PI * y);
        double u = 0.5 + 0.05 * std::cos(TWO_PI * x) * std::sin(TWO_PI * y);
        double v = 0.3 + 0.05 * std::sin(TWO_PI * x + 1.0);
        double p = 1.0 / 1.4 + 0.1 * std::cos(TWO_PI * y);
        q[0] = r;
        q[1] = r * u;
        q[2] = r * v;
        q[3] = p / (G - 1.0) + 0.5 * r * (u * u + v * v);
        return;
    }
    // manufacturedsolution.d:244-254
    q[0] = rho(x, y);
    q[1] = rho(x, y) * uu(x, y);
    q[2] = rho(x, y) * vv(x, y);
    double a = uu(x, y), b = vv(x, y);
    q[3] = pp(x, y) / (G - 1.0) + 0.5 * rho(x, y) * (a * a + b * b);
}

void mms_gradient(int kind, double x, double y, double g[4][2])
{
    if (kind == EBB_MMS_SINE) {
        double w[4], wx[4], wy[4];
        sine_prims(x, y, w, wx, wy);
        double r = w[0], u = w[1], v = w[2];
        for (int k = 0; k < 2; k++) {
            const double *d = k == 0 ? wx : wy;
            g[0][k] = d[0];
            g[1][k] = d[0] * u + r * d[1];
            g[2][k] = d[0] * v + r * d[2];
            g[3][k] = d[3] / (G - 1.0) + 0.5 * d[0] * (u * u + v * v) + r * (u * d[1] + v * d[2]);
        }
        return;
    }
    // manufacturedsolution.d:256-282
    g[0][0] = drdx(x, y);
    g[0][1] = drdy(x, y);
    g[1][0] = uu(x, y) * drdx(x, y) + rho(x, y) * dudx(x, y);
    g[1][1] = uu(x, y) * drdy(x, y) + rho(x, y) * dudy(x, y);
    g[2][0] = vv(x, y) * drdx(x, y) + rho(x, y) * dvdx(x, y);
    g[2][1] = vv(x, y) * drdy(x, y) + rho(x, y) * dvdy(x, y);
    double a = uu(x, y), b = vv(x, y);
    double dru2dx = 2.0 * rho(x, y) * uu(x, y) * dudx(x, y) + (a * a) * drdx(x, y);
    double dru2dy = 2.0 * rho(x, y) * uu(x, y) * dudy(x, y) + (a * a) * drdy(x, y);
    double drv2dx = 2.0 * rho(x, y) * vv(x, y) * dvdx(x, y) + (b * b) * drdx(x, y);
    double drv2dy = 2.0 * rho(x, y) * vv(x, y) * dvdy(x, y) + (b * b) * drdy(x, y);
    g[3][0] = 1.0 / (G - 1.0) * dpdx(x, y) + 0.5 * (dru2dx + drv2dx);
    g[3][1] = 1.0 / (G - 1.0) * dpdy(x, y) + 0.5 * (dru2dy + drv2dy);
}

void mms_source(int kind, double x, double y, const ebb_config &cfg, double mu, double S[4])
{
    if (kind == EBB_MMS_SINE) {
        double w[4], wx[4], wy[4];
        sine_prims(x, y, w, wx, wy);
        double r = w[0], u = w[1], v = w[2], p = w[3];
        double rx = wx[0], ry = wy[0], ux = wx[1], uy = wy[1], vx = wx[2], vy = wy[2], px = wx[3], py = wy[3];
        double rE = p / (G - 1.0) + 0.5 * r * (u * u + v * v);
        double rEx = px / (G - 1.0) + 0.5 * rx * (u * u + v * v) + r * (u * ux + v * vx);
        double rEy = py / (G - 1.0) + 0.5 * ry * (u * u + v * v) + r * (u * uy + v * vy);
        double H = rE + p, Hx = rEx + px, Hy = rEy + py;
        S[0] = rx * u + r * ux + ry * v + r * vy;
        S[1] = rx * u * u + 2.0 * r * u * ux + px + ry * u * v + r * uy * v + r * u * vy;
        S[2] = rx * u * v + r * ux * v + r * u * vx + ry * v * v + 2.0 * r * v * vy + py;
        S[3] = ux * H + u * Hx + vy * H + v * Hy;
        return;
    }
    // manufacturedsolution.d:158-242
    double q[4], dq[4][2];
    mms_solution(EBB_MMS_REFERENCE, x, y, q);
    mms_gradient(EBB_MMS_REFERENCE, x, y, dq);
    double r = q[0], u = q[1] / q[0], v = q[2] / q[0], ru = q[1], rv = q[2];
    double p = pressure(q);
    double ux = dudx(x, y), uy = dudy(x, y), vy = dvdy(x, y), vx = dvdx(x, y);
    double px = dpdx(x, y), py = dpdy(x, y);
    double rE = q[3];
    double Fx[4], Fy[4];
    Fx[0] = dq[1][0];
    Fx[1] = 2.0 * ru * ux + (u * u) * dq[0][0] + px;
    Fx[2] = u * v * dq[0][0] + r * u * vx + r * v * ux;
    Fx[3] = u * dq[3][0] + rE * ux + u * px + p * ux;
    Fy[0] = dq[2][1];
    Fy[1] = u * v * dq[0][1] + r * u * vy + r * v * uy;
    Fy[2] = 2.0 * rv * vy + (v * v) * dq[0][1] + py;
    Fy[3] = v * dq[3][1] + rE * vy + v * py + p * vy;
    for (int c = 0; c < 4; c++) S[c] = Fx[c] + Fy[c];
    if (cfg.viscosity) {
        double Gx[4] = {0, 0, 0, 0}, Gy[4] = {0, 0, 0, 0};
        double R = cfg.r_gas, Pr = cfg.pr;
        double k = (G * R * mu) / ((G - 1) * Pr);
        double uxx = d2udx2(x, y), uyy = d2udy2(x, y), uxy = d2udxy(x, y);
        double vxx = d2vdx2(x, y), vyy = d2vdy2(x, y), vxy = d2vdxy(x, y);
        double pxx = d2pdx2(x, y), pyy = d2pdy2(x, y), rxx = d2rdx2(x, y), ryy = d2rdy2(x, y);
        double rx = dq[0][0], ry = dq[0][1];
        Gx[1] = mu * (2.0 / 3.0) * (2 * uxx - vxy);
        Gx[2] = mu * (uxy + vxx);
        Gx[3] = mu * (2.0 / 3.0) * (2 * (u * uxx + ux * ux) - (u * vxy + ux * vy));
        Gx[3] += mu * ((v * uxy + vx * uy) + (v * vxx + vx * vx));
        double Txx = (1.0 / R) * ((1.0 / r) * pxx + (1.0 / (r * r)) * rx * px - (1.0 / (r * r * r)) * (r * px - 2.0 * p * rx) * rx -
                                  (p / (r * r)) * rxx);
        Gx[3] += k * Txx;
        Gy[1] = mu * (uyy + vxy);
        Gy[2] = mu * (2.0 / 3.0) * (2 * vyy - uxy);
        Gy[3] = mu * (2.0 / 3.0) * (2.0 * (v * vyy + vy * vy) - (v * uxy + vy * ux));
        Gy[3] += mu * (u * uyy + uy * uy + u * vxy + uy * vx);
        double Tyy = (1.0 / R) * ((1.0 / r) * pyy + (1.0 / (r * r)) * ry * py - (1.0 / (r * r * r)) * (r * py - 2.0 * p * ry) * ry -
                                  (p / (r * r)) * ryy);
        Gy[3] += k * Tyy;
        for (int c = 0; c < 4; c++) S[c] -= (Gx[c] + Gy[c]);
    }
}

}  // namespace ebb

extern "C" {

void ebb_config_defaults(ebb_config *c)
{
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->dt = 1e-5;
    c->dynamic_dt = 1;
    c->t_end = 1.0;
    c->flux = EBB_FLUX_ROE;
    c->save_iter = -1;
    c->plot_iter = -1;
    c->integrator = EBB_INT_EULER;
    c->limited = 1;
    c->lp_thresh = -1;
    c->order = 2;
    c->cfl = 0.5;
    c->ic[0] = 0.5;
    c->ic[3] = 1.0;
    c->multistage_limiting = 1;
    c->cfl_adjust = 1;
    c->pr = 0.7;
    c->r_gas = 8.3145;
    c->gamma = 1.4;
    c->mu = NAN;
    c->re = 1000;
    c->l_ref = 1;
}

int ebb_config_parse(const char *json_text, ebb_config *out, char *err, size_t err_len)
{
    if (!json_text || !out) return EBB_ERR_ARG;
    std::string e;
    if (!ebb::parse_config_json(json_text, out, e)) {
        ebb::set_err(err, err_len, e);
        return EBB_ERR_FORMAT;
    }
    return EBB_OK;
}

}  // extern "C"
