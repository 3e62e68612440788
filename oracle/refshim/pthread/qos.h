/* Stand-in for macOS <pthread/qos.h>: the QoS class request is a no-op on Linux. */
#ifndef KITE_REFSHIM_QOS_H
#define KITE_REFSHIM_QOS_H
#define QOS_CLASS_USER_INTERACTIVE 0
static inline int pthread_set_qos_class_self_np(int cls, int prio) { (void)cls; (void)prio; return 0; }
#endif
