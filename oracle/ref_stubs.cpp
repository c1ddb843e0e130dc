// ref_stubs.cpp -- stand-ins for the reference's three NetCDF-backed state-file
// classes (source/wghmStateFile.h, snowInElevationFile.h,
// additionalOutputInputFile.h), so that the reference's own translation units
// link without NetCDF.  They only hold the in-memory arrays the day loop
// writes; loading and saving files is not needed by the reference harness.
// TEST INFRASTRUCTURE ONLY: compiled solely into oracle/_ref/.
#include "wghmStateFile.h"
#include "snowInElevationFile.h"
#include "additionalOutputInputFile.h"

static const size_t kStateDays = 31;

Cell::Cell() : _cellID(0) { resize(kStateDays); }
Cell::Cell(size_t cellID, size_t l) : _cellID(cellID) { resize(l); }
Cell::Cell(const Cell &c) = default;
Cell &Cell::operator=(const Cell &c) = default;
void Cell::resize(size_t l) {
  for (auto *v : {&_canopy, &_snow, &_soil, &_locallake, &_localwetland, &_globallake, &_globalwetland,
                  &_reservoir, &_river, &_groundwater})
    v->assign(l, 0.0);
}
void Cell::lastDay_remains() {}
Cell Cell::mean() { return *this; }
double Cell::tws(int) { return 0.0; }

WghmStateFile::WghmStateFile(size_t numCells, size_t len) {
  _cells.reserve(numCells);
  for (size_t i = 0; i < numCells; i++) _cells.emplace_back(i, len ? len : kStateDays);
}
WghmStateFile::WghmStateFile(const WghmStateFile &f) = default;
WghmStateFile &WghmStateFile::operator=(const WghmStateFile &f) = default;
void WghmStateFile::load(std::string) {}
void WghmStateFile::saveMean(std::string) {}
void WghmStateFile::saveDay(std::string, int) {}
void WghmStateFile::lastDay_inplace() {}
void WghmStateFile::mean_inplace() {}
void WghmStateFile::resizeCells(size_t l) { for (auto &c : _cells) c.resize(l); }
void WghmStateFile::resetCells(size_t l) { for (auto &c : _cells) c.resize(l ? l : kStateDays); }

SnowInElevationFile::SnowInElevationFile() : _numLandCells(ng), _numLevels(101) {
  _snowInElevation.assign(ng, std::vector<double>(101, 0.0));
}
void SnowInElevationFile::load(std::string) {}
void SnowInElevationFile::save(std::string) {}

AdditionalOutputInputFile::AdditionalOutputInputFile() : additionalfilestatus(0) {
  _additionalOutputInput.assign(ng, std::vector<double>(53, 0.0));
}
void AdditionalOutputInputFile::load(std::string) {}
void AdditionalOutputInputFile::save(std::string) {}
