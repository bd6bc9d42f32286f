// Drop-in TempField (reference: src/src-mpi/TempField.h:13-36). The
// temperature of a step is evaluated on the device by cafe_sim_temperature:
// the analytic double-ellipsoid field (TempField::AnalyticTempCurr,
// TempField.C:139-217) or, when the deck selects it, the EASM field
// (TempField::EASM, TempField.C:79-137), including the end-of-scan check that
// may set Grid::inewscanflg / inewlayerflg. The field stays on the device:
// TempCurr and BuildjID are copied into these vectors by Sync(), which
// VoxelsCA::WriteToHDF1 calls (a TempOut other than TempCurr is filled at once).
// See Grid.h.
#ifndef TEMPFIELD_H
#define TEMPFIELD_H

#include <cmath>
#include <string>
#include <vector>

#include "BasePlate.h"
#include "Grid.h"
#include "Partition.h"
#include "Utilities.h"

class TempField {
 public:
  TempField(Grid &g, Partition &part, BasePlate &bp, Utilities &ut) : _xyz(&g), _part(&part), _bp(&bp), _ut(&ut) {
    Refresh();
    patternID = g.patternID;
    bmV = g.bmV;
    bmP = g.bmP;
    T0 = g.T0;
  }

  // TempField::InitializeAnalytic (TempField.C:53-77): the engine derived the
  // pool's ellipsoid axes when the Grid was created.
  void InitializeAnalytic() {}

  // TempField::AnalyticTempCurr (TempField.C:139-217) at the Grid's time
  // (main1.C passes g.time; another time is rejected) for every cell
  // (icellid is the identity at world size 1).
  void AnalyticTempCurr(double tcurr, std::vector<double> &TempOut, std::vector<int> &icellid, int Ntot) {
    if (_xyz->EASM_Flag == 1) throw std::logic_error("TempField::AnalyticTempCurr on a deck that selects EASM");
    step(tcurr, TempOut, icellid, Ntot, "TempField::AnalyticTempCurr");
  }
  // TempField::EASM (TempField.C:79-137) for a deck that selects it.
  void EASM(std::vector<double> &TempOut, std::vector<int> &icellid, int Ntot) {
    if (_xyz->EASM_Flag != 1) throw std::logic_error("TempField::EASM on a deck that does not select EASM");
    step(_xyz->time, TempOut, icellid, Ntot, "TempField::EASM");
  }

  // Extension: TempCurr and BuildjID from the device.
  void Sync() {
    const size_t n = ncell();
    TempCurr.resize(n);
    BuildjID.resize(n);
    amcafe_dropin::check(cafe_sim_download_temperature(_xyz->Engine(), TempCurr.data()), "TempField::Sync");
    amcafe_dropin::check(
        cafe_sim_download_state(_xyz->Engine(), nullptr, nullptr, nullptr, nullptr, BuildjID.data()),
        "TempField::Sync");
  }
  void Refresh() {
    cafe_grid c;
    amcafe_dropin::check(cafe_sim_grid(_xyz->Engine(), &c), "TempField");
    tInd = c.tf_tInd;
    DelT = c.DelT;
  }

  std::vector<std::vector<double>> Temp;
  std::vector<double> DDtTemp, dXM, TempCurr, lamXYZ, bmSTD, bmLx, bmX0, bmDX, bmPeriod, offset, shiftL;
  std::vector<int> nXM, nTTemp, ispvec, BuildjID;
  int NtM = 0, indexM = 0, patternID = 0, nSource = 1, tInd = 0;
  double dtM = 0, bmV = 0, bmP = 0, bmEta = 0, rcut = 0, tcut = 0, T0 = 0, Ci = 0, DelT = 0, alpha = 0, T0targ = 0,
         zlaserOff = 0, tBeg0 = 0;
  std::vector<double> a1, a2, Qp, tBeg;

 private:
  size_t ncell() const { return (size_t)_xyz->nX[0] * _xyz->nX[1] * _xyz->nX[2]; }
  void step(double tcurr, std::vector<double> &TempOut, std::vector<int> &, int Ntot, const char *where) {
    if (tcurr != _xyz->time) throw std::invalid_argument(std::string(where) + ": time must be the Grid's time");
    if ((size_t)Ntot != ncell()) throw std::invalid_argument(std::string(where) + ": Ntot must be the cell count");
    amcafe_dropin::check(cafe_sim_temperature(_xyz->Engine()), where);
    _xyz->Refresh();
    Refresh();
    if (&TempOut != &TempCurr) {
      TempOut.resize(ncell());
      amcafe_dropin::check(cafe_sim_download_temperature(_xyz->Engine(), TempOut.data()), where);
    }
  }
  Grid *_xyz;
  Partition *_part;
  BasePlate *_bp;
  Utilities *_ut;
};

#endif
