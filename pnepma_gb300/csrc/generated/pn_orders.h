// Generated by pnepma_gb300/codegen.py -- do not edit.
#pragma once
#define PN_FOR_EACH_ORDER(X) X(1) X(3) X(5) X(7) X(9) X(11)
