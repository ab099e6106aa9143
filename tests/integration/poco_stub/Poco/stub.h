// Test-only stand-ins for the part of the Poco C++ libraries that PPI's
// unchanged src/main.cc, src/ppi.cc, src/common, src/server and src/client
// name (Poco is not installed here).  Enough to compile and link PPI with the
// GB300 adapter and to run its evolution loop on one island: the TCP server
// accepts nothing, and sockets report failure if a peer is ever contacted
// (PPI runs without -peers here).  Not part of the product.
#pragma once
#include <chrono>
#include <exception>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace Poco {

class Exception : public std::exception {
public:
   explicit Exception(const std::string& msg = "Poco exception") : m_msg(msg) {}
   const char* what() const noexcept override { return m_msg.c_str(); }
   std::string displayText() const { return m_msg; }
private:
   std::string m_msg;
};

class FastMutex {
public:
   void lock() { m_m.lock(); }
   void unlock() { m_m.unlock(); }
   class ScopedLock {
   public:
      explicit ScopedLock(FastMutex& m) : m_ref(m) { m_ref.lock(); }
      ~ScopedLock() { m_ref.unlock(); }
   private:
      FastMutex& m_ref;
   };
private:
   std::mutex m_m;
};

class Runnable {
public:
   virtual ~Runnable() {}
   virtual void run() = 0;
};

class Thread {
public:
   static void sleep(long ms) { std::this_thread::sleep_for(std::chrono::milliseconds(ms)); }
};

// Runs each task on the calling thread (PPI starts one per peer).
class ThreadPool {
public:
   int available() const { return 1 << 20; }
   void addCapacity(int) {}
   void start(Runnable& r) { r.run(); }
   void stopAll() {}
   void joinAll() {}
   static ThreadPool& defaultPool() {
      static ThreadPool p;
      return p;
   }
};

class Timespan {
public:
   Timespan(long seconds = 0, long microseconds = 0) : m_us(seconds * 1000000L + microseconds) {}
private:
   long m_us;
};

template <class C>
class AutoPtr {
public:
   AutoPtr(C* p = nullptr) : m_p(p) {}
   C* operator->() const { return m_p; }
   C* get() const { return m_p; }
private:
   C* m_p;   // the channels live as long as the process (leaked on purpose)
};

class PatternFormatter {
public:
   void setProperty(const std::string&, const std::string&) {}
};
class ConsoleChannel {};
class FormattingChannel {
public:
   template <class F, class C>
   FormattingChannel(const F&, const C&) {}
};

class Logger {
public:
   static Logger& get(const std::string&) {
      static Logger l;
      return l;
   }
   void setLevel(const std::string&) {}
   template <class C>
   void setChannel(const C&) {}
   void debug(const std::string&) {}
   void information(const std::string&) {}
   void warning(const std::string&) {}
   void error(const std::string&) {}
   void fatal(const std::string&) {}
};

namespace Net {

class SocketAddress {
public:
   SocketAddress() {}
   SocketAddress(const std::string& host, int port) : m_text(host + ":" + std::to_string(port)) {}
   explicit SocketAddress(const std::string& hostport) : m_text(hostport) {}
   std::string toString() const { return m_text; }
private:
   std::string m_text;
};

class Socket {};

class StreamSocket : public Socket {
public:
   int sendBytes(const void*, int) { throw Exception("no network in this build"); }
   int receiveBytes(void*, int) { throw Exception("no network in this build"); }
   void connect(const SocketAddress&) { throw Exception("no network in this build"); }
   void connect(const SocketAddress&, const Timespan&) { throw Exception("no network in this build"); }
   void close() {}
   void shutdown() {}
};

class ServerSocket : public Socket {
public:
   explicit ServerSocket(const SocketAddress&) {}
};

class TCPServerParams {};

class TCPServerConnection : public Runnable {
public:
   explicit TCPServerConnection(const StreamSocket& s) : m_socket(s) {}
   StreamSocket& socket() { return m_socket; }
private:
   StreamSocket m_socket;
};

class TCPServerConnectionFactory {
public:
   virtual ~TCPServerConnectionFactory() {}
};

template <class S>
class TCPServerConnectionFactoryImpl : public TCPServerConnectionFactory {};

class TCPServer {
public:
   TCPServer(TCPServerConnectionFactory*, ServerSocket&, TCPServerParams*) {}
   void start() {}
};

}  // namespace Net
}  // namespace Poco

#define poco_debug(logger, msg) ((void)0)
#define poco_information(logger, msg) ((void)0)
#define poco_warning(logger, msg) ((void)0)
#define poco_error(logger, msg) ((void)0)
#define poco_fatal(logger, msg) ((void)0)
