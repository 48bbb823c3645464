/* Empty stand-in for glog: the reference includes <glog/logging.h> but never
 * calls any glog macro on the path this harness builds. Test infrastructure. */
#pragma once
