// Derived-type binary restarts of the reference (lib/io_restart_derivedtype.F90:
// write_all_bin_restarts / read_all_bin_restarts): one file per derived type
// and rank, <dir>/np<npes>/t_mesh.<rank>, t_partit.<rank>, t_tracer.<rank>,
// t_dynamics.<rank>, plus the text file <dir>/meta.time.
//
// Each file is what one Fortran `write(unit) object` statement with the
// type's WRITE(UNFORMATTED) procedure produces on a sequential unformatted
// unit (gfortran): a single record, because the procedure's own writes are
// child data transfers that continue the parent's record. A record is
// framed by 4-byte length markers before and after its bytes; longer than
// 2**31 - 9 bytes it is split into subrecords whose markers carry a minus
// sign where the record continues (leading marker) or was continued
// (trailing marker). Inside the record the fields follow the procedures'
// order (lib/MOD_MESH.F90:185-275, lib/MOD_PARTIT.F90:113-185,
// lib/MOD_TRACER.F90:104-230, lib/MOD_DYN.F90:189-300): integers and
// logicals 4 bytes (logical .true. = 1), reals 8 bytes (the double
// precision build, WP = MP = 8), character(20) blank padded, and every
// allocatable array as its extents (4-byte integers, one per dimension; all
// zero when unallocated) followed by its elements in column-major order.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace fgb {
struct HostMesh;

namespace restart {

enum class Kind { I4, R8, L4, C20, ArrI4, ArrR8 };

// One field of a record: a scalar, or an array with its extents (extents
// empty or zero: not allocated).
struct Field {
  std::string name;
  Kind kind = Kind::I4;
  int rank = 0;
  int32_t i = 0;
  double r = 0.0;
  std::string c;
  std::vector<int32_t> dims;
  std::vector<int32_t> vi;
  std::vector<double> vr;
  size_t count() const;
};

// The fields of one derived type's record, in write order.
struct Record {
  std::vector<Field> fields;
  Field* get(const std::string& name);
  const Field* get(const std::string& name) const;
  Field& add(const std::string& name, Kind kind, int rank = 0);
};

// Largest subrecord gfortran writes (2**31 - 9 bytes).
constexpr int64_t kMaxSubrecord = 2147483639LL;

// One sequential unformatted record from/to a file (subrecords joined /
// split at max_sub bytes).
bool read_record_file(const std::string& path, std::vector<uint8_t>* bytes, std::string* err);
bool write_record_file(const std::string& path, const std::vector<uint8_t>& bytes, std::string* err,
                       int64_t max_sub = kMaxSubrecord);

// Record bytes of the four types. fer_gm: the reference's Fer_GM flag
// (lib/oce_modules.F90:46, .false. by default), which adds two arrays to
// t_dynamics.
bool decode_mesh(const std::vector<uint8_t>& b, Record* out, std::string* err);
bool decode_partit(const std::vector<uint8_t>& b, Record* out, std::string* err);
bool decode_tracer(const std::vector<uint8_t>& b, Record* out, std::string* err);
bool decode_dynamics(const std::vector<uint8_t>& b, Record* out, std::string* err, bool fer_gm = false);
std::vector<uint8_t> encode(const Record& r);

// Records of a single-domain state with the reference's defaults for what
// the tracer step does not keep (unallocated arrays, the types' default
// scalars).
Record mesh_record(const HostMesh& m);
Record partit_record(int N, int M, int E);
// ntracers tracer entries with values/valuesAB (nl-1, N), schemes and the
// work arrays del_ttf, nboundary_lay, edge_up_dn_tri.
Record tracer_record(const HostMesh& m, int ntracers);
Record dynamics_record(int nl, int N, int M);

// The host mesh a t_mesh record (with the MUSCL tables of a t_tracer record,
// or none) describes; nullptr and err on inconsistent records.
HostMesh* mesh_from_records(const Record& mesh, const Record* tracer, std::string* err);

// The text file write_all_bin_restarts writes beside the np<npes> directory.
bool write_meta(const std::string& path, int cstep, int ctime, int cyear, bool tracers, bool dynamics,
                std::string* err);

}  // namespace restart
}  // namespace fgb
