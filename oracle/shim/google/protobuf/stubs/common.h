// Test-oracle support only (never linked into the product library).
//
// Minimal stand-in for the protobuf runtime header that the reference CPU
// driver includes (test_compress_cpu.cc:1) so the unmodified reference
// sources compile without libprotobuf.  It declares the one runtime entry
// point the driver calls (test_compress_cpu.cc:60) and the Message base class
// that cubelet_file.cc:29-126 serialises through.
#ifndef WL_ORACLE_SHIM_PROTOBUF_COMMON_H
#define WL_ORACLE_SHIM_PROTOBUF_COMMON_H

#include <cstdint>
#include <string>

namespace google {
namespace protobuf {

// The shim keeps no global state, so shutting the "library" down is a no-op.
inline void ShutdownProtobufLibrary() {}

// Abstract message: the three calls cubelet_file.cc makes on a message.
class Message {
 public:
  virtual ~Message() {}
  virtual int ByteSize() const = 0;
  virtual bool SerializeToArray(void *data, int size) const = 0;
  virtual bool ParseFromArray(const void *data, int size) = 0;
};

}  // namespace protobuf
}  // namespace google

#endif
