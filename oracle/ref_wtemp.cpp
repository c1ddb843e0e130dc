// ref_wtemp.cpp -- runs the reference's own calcWaterTempClass::calcWTemp
// (source/calcWaterTemp.cpp) on records read from stdin and writes its 12
// results per record to stdout.
//
// TEST INFRASTRUCTURE ONLY.  Built from the reference sources by oracle/Makefile
// (target "ref") into oracle/_ref/; it pins the C restatement (wg_wtemp.c)
// through tests/golden/wtemp_cases.npz.  A record is 73 doubles in the order of
// calcWaterTempClass::transfer (calcWaterTemp.h:23-95), the flags as 0/1.
#include <cstdio>
#include <vector>

#include "calcWaterTemp.h"

int main() {
  double r[73];
  calcWaterTempClass cwt;
  while (fread(r, sizeof(double), 73, stdin) == 73) {
    calcWaterTempClass::transfer &t = cwt.tsf;
    const double *p = r;
    t.calcTempPP = *p++ != 0.;
    t.powerPlantWW = *p++;
    t.powerPlantWC = *p++;
    t.ShortRad = *p++;
    t.LongRad = *p++;
    t.AirTempC = *p++;
    t.CellCorrFact = *p++;
    t.openWaterPET = *p++;
    t.openWaterPrecip = *p++;
    t.CellArea = *p++;
    t.GWTemp = *p++;
    t.cellInflows.assign(p, p + 9);
    p += 9;
    t.cellInflowsTemp.assign(p, p + 9);
    p += 9;
    t.iceThickness.assign(p, p + 6);
    p += 6;
    t.RiverStor = *p++;
    t.localGWRunoffIntoRiver = *p++;
    t.localRunoffIntoRiver = *p++;
    t.RiverBottomWidth = *p++;
    t.RiverLength = *p++;
    t.RiverLengthCheck = *p++;
    t.RiverInflow = *p++;
    t.hasOutflow = *p++ != 0.;
    t.locLakeArea = *p++;
    t.locLakeStorPrevStep = *p++;
    t.locLakeTempPrevStep = *p++;
    t.dailyLocLakeEvapo = *p++;
    t.locLakeAreaRedFactor = *p++;
    t.localRunoff = *p++;
    t.localGWRunoff = *p++;
    t.locWetlandArea = *p++;
    t.locWetlandStorPrevStep = *p++;
    t.locWetlandTempPrevStep = *p++;
    t.dailyLocWetlandEvapo = *p++;
    t.locWetlandAreaRedFactor = *p++;
    t.inflowLocWetland = *p++;
    t.outflowLocWetland = *p++;
    t.gloLakeArea = *p++;
    t.gloLakeStorPrevStep = *p++;
    t.gloLakeTempPrevStep = *p++;
    t.dailyGloLakeEvapo = *p++;
    t.inflowGloLake = *p++;
    t.inflowReservoir = *p++;
    t.reservoirArea = *p++;
    t.reservoirStorPrevStep = *p++;
    t.reservoirTempPrevStep = *p++;
    t.dailyReservoirEvapo = *p++;
    t.gloWetlandInflow = *p++;
    t.gloWetlandArea = *p++;
    t.gloWetlandStorPrevStep = *p++;
    t.gloWetlandTempPrevStep = *p++;
    t.dailyGloWetlandEvapo = *p++;
    t.gloWetlandAreaReductionFactor = *p++;
    if (p - r != 73) return 3;
    std::vector<double> out = cwt.calcWTemp(t);
    fwrite(out.data(), sizeof(double), 12, stdout);
  }
  return 0;
}
