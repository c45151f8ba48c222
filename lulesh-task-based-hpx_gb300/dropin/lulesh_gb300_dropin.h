// lulesh_gb300_dropin.h - the GB300 step in place of the reference's
// LagrangeLeapFrogWithTasks(Domain&) (lulesh.cc:1977-2240).
//
// Include after the reference's own "lulesh.h" in its lulesh.cc. It needs no
// change to lulesh.h: every array comes from a public Domain accessor
// (lulesh.h:281-392), and the node -> corner CSR starts, which Domain keeps
// private, are rebuilt from nodeElemCornerList(i) - nodeElemCornerList(0)
// (lulesh.h:354-355).
//
// In hpx_main (lulesh.cc:2361-2386), after the Domain is built:
//
//     LuleshGb300 gpu;
//     if (gpu.attach(*locDom, LULESH_FP64) != LULESH_OK) exit(-1);
//     while ((locDom->time() < locDom->stoptime()) && (locDom->cycle() < opts.its)) {
//         TimeIncrement(*locDom);
//         if (gpu.leapfrog(*locDom) == LULESH_EVOLUME) exit(VolumeError);  // was LagrangeLeapFrogWithTasks
//         ... progress output unchanged ...
//     }
//
// leapfrog() uploads the state a step reads from the Domain's arrays, runs
// the cycle on the GPU and downloads every field the step writes, so the rest
// of the program (progress output, VerifyAndWriteFinalOutput, the CSV line)
// reads the Domain as before.
#pragma once

#include <vector>

#include "lulesh_gb300.h"

class LuleshGb300 {
public:
    LuleshGb300() = default;
    LuleshGb300(const LuleshGb300&) = delete;
    LuleshGb300& operator=(const LuleshGb300&) = delete;
    ~LuleshGb300() {
        if (dev_) lulesh_dev_destroy(dev_);
    }

    // A view of the Domain's arrays (raw pointers, no copies) and the CSR
    // starts it needs; the Domain must outlive this object.
    static void make_view(Domain& d, std::vector<Index_t>& node_elem_start, lulesh_time_state* ts,
                          lulesh_domain_view& v) {
        v = lulesh_domain_view{};
        v.numElem = d.numElem();
        v.numNode = d.numNode();
        v.sizeX = d.sizeX();
        v.numReg = d.numReg();
        v.cost = d.cost();
        const Index_t nbc = (d.sizeX() + 1) * (d.sizeX() + 1);
        v.numSymmX = d.symmXempty() ? 0 : nbc;
        v.numSymmY = d.symmYempty() ? 0 : nbc;
        v.numSymmZ = d.symmZempty() ? 0 : nbc;
        v.x = d.x_begin();
        v.y = d.y_begin();
        v.z = d.z_begin();
        v.xd = d.xd_begin();
        v.yd = d.yd_begin();
        v.zd = d.zd_begin();
        v.xdd = d.xdd_begin();
        v.ydd = d.ydd_begin();
        v.zdd = d.zdd_begin();
        v.fx = d.fx_begin();
        v.fy = d.fy_begin();
        v.fz = d.fz_begin();
        v.nodalMass = d.nodalMass_begin();
        v.symmX = d.symmXempty() ? nullptr : d.symmX_begin();
        v.symmY = d.symmYempty() ? nullptr : d.symmY_begin();
        v.symmZ = d.symmZempty() ? nullptr : d.symmZ_begin();
        v.nodelist = d.nodelist(0);
        v.lxim = &d.lxim(0);
        v.lxip = &d.lxip(0);
        v.letam = &d.letam(0);
        v.letap = &d.letap(0);
        v.lzetam = &d.lzetam(0);
        v.lzetap = &d.lzetap(0);
        v.elemBC = &d.elemBC(0);
        v.e = &d.e(0);
        v.p = d.p_begin();
        v.q = d.q_begin();
        v.ql = &d.ql(0);
        v.qq = &d.qq(0);
        v.v = d.v_begin();
        v.vnew = d.vnew_begin();
        v.delv = &d.delv(0);
        v.vdov = d.vdov_begin();
        v.arealg = &d.arealg(0);
        v.ss = d.ss_begin();
        v.volo = &d.volo(0);
        v.elemMass = d.elemMass_begin();
        // CSR starts relative to the corner list's first entry
        const Index_t nn = d.numNode();
        node_elem_start.resize(size_t(nn) + 1);
        const Index_t* base = d.nodeElemCornerList(0);
        for (Index_t i = 0; i < nn; ++i) node_elem_start[i] = Index_t(d.nodeElemCornerList(i) - base);
        node_elem_start[nn] = node_elem_start[nn - 1] + d.nodeElemCount(nn - 1);
        v.nodeElemStart = node_elem_start.data();
        v.nodeElemCornerList = base;
        v.regNumList = d.regNumList();
        v.params = lulesh_params{d.e_cut(), d.p_cut(), d.q_cut(), d.v_cut(), d.u_cut(),
                                 d.hgcoef(), d.ss4o3(), d.qstop(), d.monoq_max_slope(),
                                 d.monoq_limiter_mult(), d.qlc_monoq(), d.qqc_monoq(), d.qqc(),
                                 d.eosvmax(), d.eosvmin(), d.pmin(), d.emin(), d.dvovmax(),
                                 d.refdens()};
        v.time = ts;
    }

    // The Domain's time-control fields (lulesh.h:563-572) as the library's
    // time state.
    static lulesh_time_state time_of(Domain& d) {
        lulesh_time_state t{};
        t.time = d.time();
        t.deltatime = d.deltatime();
        t.dtcourant = d.dtcourant();
        t.dthydro = d.dthydro();
        t.dtfixed = d.dtfixed();
        t.deltatimemultlb = d.deltatimemultlb();
        t.deltatimemultub = d.deltatimemultub();
        t.dtmax = d.dtmax();
        t.stoptime = d.stoptime();
        t.cycle = d.cycle();
        return t;
    }

    // Creates the device handle for this Domain (uploads the whole state).
    int attach(Domain& d, int32_t precision) {
        if (dev_) return LULESH_EINVAL;
        time_ = time_of(d);
        make_view(d, node_elem_start_, &time_, view_);
        return lulesh_dev_create(&view_, precision, &dev_);
    }

    // One LagrangeLeapFrog cycle with the Domain's current deltatime: the
    // drop-in for LagrangeLeapFrogWithTasks(d). On LULESH_EVOLUME (where the
    // reference exits with VolumeError) the Domain holds the partly advanced
    // state.
    int leapfrog(Domain& d) {
        if (!dev_) return LULESH_EINVAL;
        time_.deltatime = d.deltatime();
        const int st = lulesh_leapfrog(dev_, &view_);
        if (st == LULESH_OK) {
            d.dtcourant() = time_.dtcourant;
            d.dthydro() = time_.dthydro;
        }
        return st;
    }

    const lulesh_domain_view& view() const { return view_; }
    lulesh_dev* device() const { return dev_; }

private:
    lulesh_dev* dev_ = nullptr;
    lulesh_domain_view view_{};
    lulesh_time_state time_{};
    std::vector<Index_t> node_elem_start_;
};
