// TensorFlow header stand-in for the executed-reference checker.
#pragma once
#include "ctref_tf.h"
