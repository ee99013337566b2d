set output "hist_cfg1_MOTIF00018.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-79.9869:20.8483]
set yrange [0:2577]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00018.dat" using 1:2 title 'MOTIF00018 (cfg1)' with boxes
