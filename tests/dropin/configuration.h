// Minimal stand-in for the reference's inc/configuration.h: only what the drop-in
// adapter needs (TYPE is double, inc/configuration.h:20-22).  Test infrastructure.
#ifndef DROPIN_CONFIGURATION_H
#define DROPIN_CONFIGURATION_H
#define TYPE double
#endif
