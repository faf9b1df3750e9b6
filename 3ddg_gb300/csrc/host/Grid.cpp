// Grid / Block / Element facade over the C ABI; see Grid.h.
#include "Grid.h"

#include <cmath>
#include <cstring>
#include <iostream>
#include <sstream>
#include <stdexcept>

#include "Basis.h"

namespace dgfacade {

struct Sim {
    dg_handle* h = nullptr;
    dg_params p{};
    int X = 0, Y = 0, Z = 0;
    std::vector<double> rho, vel, coords;  // host mirror [X][Y][Z], [3][X][Y][Z]
    bool coords_valid = false;
    Matrix mass, stiff;                    // unit-interval M and S the simulation was created with
    ~Sim()
    {
        if (h) dg_destroy(h);
    }
    size_t gsize() const { return (size_t)X * Y * Z; }
    void check(int rc, const char* what) const
    {
        if (rc != DG_OK) throw std::runtime_error(std::string(what) + ": " + dg_last_error());
    }
    void ensure_mirror()
    {
        if (rho.size() != gsize()) {
            rho.assign(gsize(), 0.0);
            vel.assign(3 * gsize(), 0.0);
        }
    }
};

}  // namespace dgfacade

using dgfacade::Sim;

namespace {

dg_params params_from(BCParam* bc, unsigned short order, unsigned* nb, unsigned* ne, const double* w,
                      const double* c, double rho0, double c0, double ba, double diff, bool adv, bool dif,
                      bool sponge)
{
    dg_params p;
    dg_params_default(&p);
    p.order = order;
    for (int a = 0; a < 3; a++) {
        p.num_blocks[a] = (int)nb[a];
        p.num_elements[a] = (int)ne[a];
        p.elem_width[a] = w[a];
        p.corner[a] = c[a];
        p.periodic[a] = bc->IS_PERIODIC[a] ? 1 : 0;
    }
    p.rho0 = rho0;
    p.c0 = c0;
    p.b_over_a = ba;
    p.diff_const = diff;
    p.eval_advect = adv;
    p.eval_diff = dif;
    p.eval_sponge = sponge;
    p.sigma_max = bc->sigmaMax;
    for (int f = 0; f < 6; f++) p.sponge_width[f] = (int)bc->spongeWidth[f];
    p.ic_gauss[0] = bc->IC_X_GAUSS;
    p.ic_gauss[1] = bc->IC_Y_GAUSS;
    p.ic_gauss[2] = bc->IC_Z_GAUSS;
    p.ic_drho_amp = bc->IC_drho_amplitude;
    p.ic_v_amp[0] = bc->IC_vx_amplitude;
    p.ic_v_amp[1] = bc->IC_vy_amplitude;
    p.ic_v_amp[2] = bc->IC_vz_amplitude;
    p.ic_sigma = bc->IC_sigma;
    p.ic_center[0] = bc->IC_center_x;
    p.ic_center[1] = bc->IC_center_y;
    p.ic_center[2] = bc->IC_center_z;
    return p;
}

}  // namespace

// ----------------------------------------------------------------- Element
Element::Element(std::shared_ptr<Sim> s, int block, const int local[3]) : sim(std::move(s)), mBlock(block)
{
    const dg_params& p = sim->p;
    int b[3] = {block / (p.num_blocks[1] * p.num_blocks[2]), (block / p.num_blocks[2]) % p.num_blocks[1],
                block % p.num_blocks[2]};
    for (int a = 0; a < 3; a++) {
        mLocal[a] = local[a];
        mGlobal[a] = b[a] * p.num_elements[a] + local[a] - 1;
    }
}

bool Element::isHalo() const
{
    for (int a = 0; a < 3; a++)
        if (mLocal[a] == 0 || mLocal[a] == sim->p.num_elements[a] + 1) return true;
    return false;
}

string Element::getName() const
{
    std::ostringstream o;
    const dg_params& p = sim->p;
    long long addr = (long long)mBlock * (p.num_elements[0] + 2) * (p.num_elements[1] + 2) * (p.num_elements[2] + 2) +
                     ((long long)mLocal[0] * (p.num_elements[1] + 2) + mLocal[1]) * (p.num_elements[2] + 2) + mLocal[2];
    o << "EL" << addr << ":" << mGlobal[0] << "," << mGlobal[1] << "," << mGlobal[2];
    return o.str();
}

string Element::getLocalName() const
{
    std::ostringstream o;
    o << "(" << mLocal[0] - 1 << "," << mLocal[1] - 1 << "," << mLocal[2] - 1 << ")";
    return o.str();
}

unsigned short int Element::getOrder() const { return (unsigned short)sim->p.order; }

long long Element::node_offset(const int idx[3]) const
{
    if (isHalo()) return -1;
    const int K = sim->p.order + 1;
    long long ii = (long long)mGlobal[0] * K + idx[0], jj = (long long)mGlobal[1] * K + idx[1],
              kk = (long long)mGlobal[2] * K + idx[2];
    return (ii * sim->Y + jj) * sim->Z + kk;
}

double Element::getOutputRho(int idx[3]) const
{
    long long o = node_offset(idx);
    return (o < 0 || sim->rho.empty()) ? 0.0 : sim->rho[o];
}

double* Element::getOutputVelocity(int idx[3])
{
    long long o = node_offset(idx);
    for (int a = 0; a < 3; a++) mVelTmp[a] = (o < 0 || sim->vel.empty()) ? 0.0 : sim->vel[a * sim->gsize() + o];
    return mVelTmp;
}

double* Element::getOutputCoords(int idx[3])
{
    long long o = node_offset(idx);
    if (!sim->coords_valid) {
        sim->coords.assign(3 * sim->gsize(), 0.0);
        sim->check(dg_get_grid(sim->h, sim->coords.data(), nullptr), "dg_get_grid");
        sim->coords_valid = true;
    }
    for (int a = 0; a < 3; a++) mCoordTmp[a] = o < 0 ? 0.0 : sim->coords[a * sim->gsize() + o];
    return mCoordTmp;
}

double Element::getRho0() const { return sim->p.rho0; }
double Element::getC0() const { return sim->p.c0; }
double Element::getBoverA() const { return sim->p.b_over_a; }
double Element::getDiffusionConstant() const { return sim->p.diff_const; }

double Element::getSigmaU() const
{
    // sigma depends only on the element; read it from node (0,0,0)
    if (isHalo()) return 0.0;
    std::vector<double> sg(sim->gsize());
    sim->check(dg_get_grid(sim->h, nullptr, sg.data()), "dg_get_grid");
    int idx[3] = {0, 0, 0};
    return sg[node_offset(idx)];
}

void Element::setRho(int idx[3], double rho)
{
    long long o = node_offset(idx);
    sim->ensure_mirror();
    if (o >= 0) sim->rho[o] = rho;
}

void Element::setVelocityComponent(int idx[3], int axis, double v)
{
    long long o = node_offset(idx);
    sim->ensure_mirror();
    if (o >= 0) sim->vel[axis * sim->gsize() + o] = v;
}

// ----------------------------------------------------------------- Block
Block::Block(std::shared_ptr<Sim> s, int index) : sim(std::move(s)), mIndex(index)
{
    const dg_params& p = sim->p;
    mGlobalPosition[0] = index / (p.num_blocks[1] * p.num_blocks[2]);
    mGlobalPosition[1] = (index / p.num_blocks[2]) % p.num_blocks[1];
    mGlobalPosition[2] = index % p.num_blocks[2];
    for (int i = 0; i < p.num_elements[0] + 2; i++) {
        vector<vector<Element>> plane;
        for (int j = 0; j < p.num_elements[1] + 2; j++) {
            vector<Element> line;
            line.reserve(p.num_elements[2] + 2);
            for (int k = 0; k < p.num_elements[2] + 2; k++) {
                int l[3] = {i, j, k};
                line.emplace_back(sim, index, l);
            }
            plane.push_back(std::move(line));
        }
        mElements.push_back(std::move(plane));
    }
}

string Block::getName() const
{
    std::ostringstream o;
    o << "B" << mIndex << ":" << mGlobalPosition[0] << "," << mGlobalPosition[1] << "," << mGlobalPosition[2];
    return o.str();
}

string Block::getLayout() const
{
    std::string ret = getName() + "\n";
    for (size_t k = 0; k < mElements[0][0].size(); k++) {
        ret += "   k=" + std::to_string((int)k - 1) + "\n";
        for (size_t i = 0; i < mElements.size(); i++) {
            ret += "      ";
            for (size_t j = 0; j < mElements[i].size(); j++) ret += mElements[i][j][k].getName() + "   ";
            ret += "\n";
        }
    }
    return ret;
}

void Block::setZero()
{
    // zeroes this block's part of the host mirror (upload with Grid::syncToDevice)
    sim->ensure_mirror();
    int idx[3];
    for (auto& pl : mElements)
        for (auto& ln : pl)
            for (auto& e : ln) {
                if (e.isHalo()) continue;
                const int K = sim->p.order + 1;
                for (idx[0] = 0; idx[0] < K; idx[0]++)
                    for (idx[1] = 0; idx[1] < K; idx[1]++)
                        for (idx[2] = 0; idx[2] < K; idx[2]++) {
                            e.setRho(idx, 0.0);
                            for (int a = 0; a < 3; a++) e.setVelocityComponent(idx, a, 0.0);
                        }
            }
}

// ----------------------------------------------------------------- Grid
void Grid::init(const dg_params& p, const string& matrixFilename, Basis* basisPtr)
{
    sim = std::make_shared<Sim>();
    sim->p = p;
    const char* mf = matrixFilename.empty() ? nullptr : matrixFilename.c_str();
    const char* cf = (basisPtr && !basisPtr->coeffFile().empty()) ? basisPtr->coeffFile().c_str() : nullptr;
    sim->check(dg_create(&p, mf, cf, &sim->h), "dg_create");
    sim->check(dg_dims(sim->h, &sim->X, &sim->Y, &sim->Z), "dg_dims");
    const int K = p.order + 1;
    std::vector<double> m((size_t)K * K), st((size_t)K * K);
    sim->check(dg_line_operators(p.order, p.lumped_mass, mf, cf, m.data(), st.data(), nullptr, nullptr, nullptr,
                                 nullptr),
               "dg_line_operators");
    sim->mass = Matrix(K, K, m.data());
    sim->stiff = Matrix(K, K, st.data());
    mOrder = p.order;
    for (int a = 0; a < 3; a++) {
        mNumElements[a] = p.num_elements[a];
        mNumBlocks[a] = p.num_blocks[a];
    }
    build_views();
}

void Grid::build_views()
{
    mBlocks.clear();
    int b = 0;
    for (int i = 0; i < mNumBlocks[0]; i++) {
        vector<vector<Block>> plane;
        for (int j = 0; j < mNumBlocks[1]; j++) {
            vector<Block> line;
            for (int k = 0; k < mNumBlocks[2]; k++) line.emplace_back(sim, b++);
            plane.push_back(std::move(line));
        }
        mBlocks.push_back(std::move(plane));
    }
}

Grid::Grid(string matrixFilename, BCParam* BCP, unsigned short int order, unsigned int* numBlocks,
           unsigned int* numElem, float* elemWidth, float* startingCorner, Basis* basisPtr, float Rho0, float C0,
           float BoverA, float Mu_visc, bool evalAdvect, bool evalDiff, bool evalSponge)
{
    double w[3], c[3];
    for (int a = 0; a < 3; a++) {
        w[a] = elemWidth[a];
        c[a] = startingCorner[a];
    }
    init(params_from(BCP, order, numBlocks, numElem, w, c, Rho0, C0, BoverA, Mu_visc, evalAdvect, evalDiff,
                     evalSponge),
         matrixFilename, basisPtr);
}

Grid::Grid(string matrixFilename, BCParam* BCP, unsigned short int order, unsigned int* numBlocks,
           unsigned int* numElem, double* elemWidth, double* startingCorner, Basis* basisPtr, double Rho0, double C0,
           double BoverA, double Mu_visc, bool evalAdvect, bool evalDiff, bool evalSponge)
{
    init(params_from(BCP, order, numBlocks, numElem, elemWidth, startingCorner, Rho0, C0, BoverA, Mu_visc,
                     evalAdvect, evalDiff, evalSponge),
         matrixFilename, basisPtr);
}

Grid::Grid(const dg_params& p, string matrixFilename, Basis* basisPtr) { init(p, matrixFilename, basisPtr); }

Grid::Grid(const Grid& g) : mBlocks(g.mBlocks), sim(g.sim), mOrder(g.mOrder)
{
    for (int a = 0; a < 3; a++) {
        mNumElements[a] = g.mNumElements[a];
        mNumBlocks[a] = g.mNumBlocks[a];
    }
}

Grid& Grid::operator=(const Grid& g)
{
    sim = g.sim;
    mBlocks = g.mBlocks;
    mOrder = g.mOrder;
    for (int a = 0; a < 3; a++) {
        mNumElements[a] = g.mNumElements[a];
        mNumBlocks[a] = g.mNumBlocks[a];
    }
    return *this;
}

void Grid::RK33(double dt, Grid* oldGrid, Grid* k1, Grid* k2, ofstream& logFile)
{
    (void)k1;
    (void)k2;
    (void)logFile;
    if (oldGrid && oldGrid->sim != sim)
        throw std::invalid_argument("Grid::RK33: oldGrid is a different simulation (not a copy of this Grid)");
    sim->check(dg_step(sim->h, dt, 1), "dg_step");
}

void Grid::setZero()
{
    sim->rho.assign(sim->gsize(), 0.0);
    sim->vel.assign(3 * sim->gsize(), 0.0);
    syncToDevice();
}

void Grid::syncToHost()
{
    sim->ensure_mirror();
    sim->check(dg_get_state(sim->h, sim->rho.data(), sim->vel.data()), "dg_get_state");
}

void Grid::syncToDevice()
{
    sim->ensure_mirror();
    sim->check(dg_set_state(sim->h, sim->rho.data(), sim->vel.data()), "dg_set_state");
}

dg_handle* Grid::handle() { return sim->h; }

Matrix* Grid::getMass() { return &sim->mass; }

Matrix* Grid::getStiff() { return &sim->stiff; }

double Grid::time() const { return dg_time(sim->h); }

string Grid::getLayout()
{
    string ret;
    for (auto& pl : mBlocks)
        for (auto& ln : pl)
            for (auto& b : ln) ret += b.getLayout() + "\n";
    return ret;
}

string Grid::allDRhoToString(bool twoDOnly)
{
    syncToHost();
    std::ostringstream o;
    o.setf(std::ios::fixed);
    o.precision(15);
    for (size_t bi = 0; bi < mBlocks.size(); bi++)
        for (size_t bj = 0; bj < mBlocks[bi].size(); bj++)
            for (size_t bk = 0; bk < mBlocks[bi][bj].size(); bk++) {
                if (twoDOnly && bk != 0) continue;
                o << "Block " << bi << "," << bj << "," << bk << "\n";
                Block& b = mBlocks[bi][bj][bk];
                for (size_t i = 0; i < b.mElements.size(); i++)
                    for (size_t j = 0; j < b.mElements[i].size(); j++)
                        for (size_t k = 0; k < b.mElements[i][j].size(); k++) {
                            if (twoDOnly && k != 1) continue;
                            Element& e = b.mElements[i][j][k];
                            o << "   Elem " << i << "," << j << "," << k << "\n";
                            const int K = mOrder + 1;
                            int idx[3];
                            for (idx[0] = 0; idx[0] < K; idx[0]++)
                                for (idx[1] = 0; idx[1] < K; idx[1]++)
                                    for (idx[2] = 0; idx[2] < K; idx[2]++) {
                                        if (twoDOnly && idx[2] != 0) continue;
                                        o << "      Node " << idx[0] << "," << idx[1] << "," << idx[2] << ": "
                                          << e.getOutputRho(idx) << "\n";
                                    }
                        }
            }
    return o.str();
}
